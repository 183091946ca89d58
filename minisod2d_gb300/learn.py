"""Entropy-viscosity estimators: plain and learned (host orchestration over the C ABI).

The plain estimator (``entropy_viscosity``) and the learned one
(``Mlp`` + ``learned_viscosity``) produce the per-element artificial
viscosity nu_e; the diffusion residual consumes mu_e(e, a) = rho(a) nu_e
either as the reference's mu_e(nelem, ngaus) array (``full_diffusion_ijk``) or
directly per element (``diffusion_ijk_nu``).  Training data are feature ->
y = nu / nu_max pairs generated by the plain estimator on seeded shock-like
fields.
"""
import ctypes as C
import os

import numpy as np

from . import capi, workload

GAMMA, RGAS, CE, CMAX = 1.4, 287.0, 0.1, 0.5
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def shipped_weights(workload_name):
    """Weight file of the network trained on a workload (python -m minisod2d_gb300.learn writes them)."""
    return os.path.join(DATA, "mlp_%s.bin" % workload_name)


def shipped_report(workload_name):
    import json

    with open(os.path.join(DATA, "%s_report.json" % workload_name)) as f:
        return json.load(f)


# Network trained on the learned_48 workload (48^3 hexes, porder 4, shock-like
# fields, 64 training seeds).  The features and the target depend on the mesh
# size and the order, so each workload has its own network.
SHIPPED_WEIGHTS = shipped_weights("learned_48")
NFEAT = 12
NPARAMS = 1505


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(stream):
    if stream is not None:
        return stream
    import torch

    return torch.cuda.current_stream().cuda_stream


def _geo(dev):
    return [dev.cfg.porder, dev.nelem, dev.npoin, _p(dev.connec), _p(dev.He), _p(dev.gpvol), _p(dev.dlxigp_ip),
            _p(dev.invAtoIJK), _p(dev.AtoI), _p(dev.AtoJ), _p(dev.AtoK)]


def entropy_viscosity(dev, mu_e=None, nu=None, numax=None, ce=CE, cmax=CMAX, gamma=GAMMA, normalise=True,
                      stream=None):
    """Plain estimator on a DeviceCase: writes mu_e (nelem*nnode) and returns (mu_e, nu, numax)."""
    import torch

    n = dev.cfg.nnode
    mu_e = mu_e if mu_e is not None else torch.empty(dev.nelem * n, device=dev.rho.device)
    nu = nu if nu is not None else torch.empty(dev.nelem, device=dev.rho.device)
    numax = numax if numax is not None else torch.empty(dev.nelem, device=dev.rho.device)
    capi.call("msod_entropy_viscosity", *_geo(dev), _p(dev.rho), _p(dev.u), _p(dev.pr), float(gamma), float(ce),
              float(cmax), 1 if normalise else 0, _p(mu_e), _p(nu), _p(numax), _stream(stream))
    return mu_e, nu, numax


def features(dev, feat=None, numax=None, cmax=CMAX, gamma=GAMMA, stream=None):
    import torch

    feat = feat if feat is not None else torch.empty(dev.nelem * NFEAT, device=dev.rho.device)
    numax = numax if numax is not None else torch.empty(dev.nelem, device=dev.rho.device)
    capi.call("msod_mlp_features", *_geo(dev), _p(dev.rho), _p(dev.u), _p(dev.pr), 0.0, float(gamma), float(cmax),
              _p(feat), _p(numax), _stream(stream))
    return feat, numax


class Mlp:
    """The per-element network (device weights behind an opaque handle)."""

    def __init__(self, seed=0):
        self.h = C.c_void_p()
        capi.call("msod_mlp_create", C.byref(self.h), int(seed))

    def __del__(self):
        try:
            if self.h:
                capi.lib().msod_mlp_destroy(self.h)
        except Exception:
            pass

    def train(self, feat, target, steps=2000, batch=4096, lr=1e-3, seed=0, weight=None, stream=None):
        n = target.numel()
        loss = np.zeros(steps, np.float32)
        capi.call("msod_mlp_train", self.h, _p(feat), _p(target), _p(weight), int(n), int(steps), int(batch),
                  float(lr), int(seed), loss.ctypes.data_as(C.c_void_p), _stream(stream))
        return loss

    def gradient(self, feat, target, idx, weight=None, stream=None):
        g = np.zeros(NPARAMS, np.float32)
        capi.call("msod_mlp_gradient", self.h, _p(feat), _p(target), _p(weight), _p(idx), int(idx.numel()),
                  g.ctypes.data_as(C.c_void_p), _stream(stream))
        return g

    def params(self):
        w = np.zeros(NPARAMS, np.float32)
        nm = np.zeros(4 * NFEAT, np.float32)
        capi.call("msod_mlp_get_params", self.h, w.ctypes.data_as(C.c_void_p), nm.ctypes.data_as(C.c_void_p))
        return w, nm

    def set_params(self, w=None, norm=None):
        w = None if w is None else np.ascontiguousarray(w, np.float32)
        norm = None if norm is None else np.ascontiguousarray(norm, np.float32)
        capi.call("msod_mlp_set_params", self.h, w.ctypes.data_as(C.c_void_p) if w is not None else None,
                  norm.ctypes.data_as(C.c_void_p) if norm is not None else None)

    def predict(self, feat, numax=None, stream=None):
        import torch

        ne = feat.numel() // NFEAT
        y = torch.empty(ne, device=feat.device)
        nu = torch.empty(ne, device=feat.device) if numax is not None else None
        flag = torch.empty(ne, dtype=torch.int32, device=feat.device)
        capi.call("msod_mlp_predict", self.h, _p(feat), _p(numax), int(ne), _p(y), _p(nu), _p(flag),
                  _stream(stream))
        return y, nu, flag

    def save(self, path):
        capi.call("msod_mlp_save", self.h, os.fsencode(path))

    def load(self, path):
        capi.call("msod_mlp_load", self.h, os.fsencode(path))


def learned_viscosity(mlp, dev, nu=None, flag=None, ce=CE, cmax=CMAX, gamma=GAMMA, stream=None):
    """nu_e per element from the network, with the plain estimator on out-of-range elements."""
    import torch

    nu = nu if nu is not None else torch.empty(dev.nelem, device=dev.rho.device)
    flag = flag if flag is not None else torch.empty(dev.nelem, dtype=torch.int32, device=dev.rho.device)
    capi.call("msod_learned_viscosity", mlp.h, *_geo(dev), _p(dev.rho), _p(dev.u), _p(dev.pr), 0.0, float(gamma),
              float(ce), float(cmax), _p(nu), _p(flag), _stream(stream))
    return nu, flag


def diffusion_learned(mlp, dev, out=None, nu=None, flag=None, ce=CE, cmax=CMAX, gamma=GAMMA, from_T=False,
                      stream=None):
    """Diffusion with the learned viscosity in one call (msod_diffusion_ijk_learned:
    the learned viscosity -- features from rho, u and the pressure, or
    p = rho Rgas T with ``from_T``; plain-estimator fallback per element --
    then the per-element-viscosity diffusion).  Returns the residuals, the
    viscosity used and the fallback flags."""
    import torch

    out = out or (dev.Dmass, dev.Dmom, dev.Dener)
    nu = nu if nu is not None else torch.empty(dev.nelem, device=dev.rho.device)
    flag = flag if flag is not None else torch.empty(dev.nelem, dtype=torch.int32, device=dev.rho.device)
    capi.call("msod_diffusion_ijk_learned", mlp.h, *_geo(dev), float(dev.cfg.Cp), float(dev.cfg.Pr), _p(dev.rho),
              _p(dev.u), _p(dev.Tem), _p(dev.mu_fluid), _p(dev.mu_sgs), _p(dev.Tem if from_T else dev.pr),
              float(RGAS if from_T else 0.0), float(gamma), float(ce), float(cmax), *[_p(o) for o in out], _p(nu),
              _p(flag), _stream(stream))
    return out, nu, flag


def diffusion_ijk_nu(dev, nu, out=None, stream=None):
    """Diffusion residual with mu_e(e, a) = rho(a) nu(e)."""
    out = out or (dev.Dmass, dev.Dmom, dev.Dener)
    capi.call("msod_diffusion_ijk_nu", *_geo(dev), float(dev.cfg.Cp), float(dev.cfg.Pr), _p(dev.rho), _p(dev.u),
              _p(dev.Tem), _p(dev.mu_fluid), _p(nu), _p(dev.mu_sgs), *[_p(o) for o in out], _stream(stream))
    return out


def loss_weights(y, numax, feat, share):
    """Per-sample weights of the training loss (mean 1): a uniform part 1 - share and a part
    `share` proportional to (nu * J)^2, nu = y nu_max the plain estimator's viscosity and J the
    element's relative density jump (feature 0 is its logarithm).  The artificial mass
    diffusion nu_e div grad rho (elem_diffu.f90:183) is set almost entirely by the few shock
    elements with the largest nu J; a decade error there costs Rmass in proportion to nu J, while
    the uniform part keeps the fit of every decade."""
    import torch

    if share <= 0.0:
        return None
    jump = torch.exp(feat.view(-1, NFEAT)[:, 0].double())
    m = (y.double() * numax.double() * jump) ** 2
    m = m / torch.clamp(m.mean(), min=1e-300)
    return ((1.0 - share) + share * m).float().contiguous()


def training_data(cfg, seeds, device="cuda", with_numax=False):
    """Features and targets y = nu / nu_max of the plain estimator over seeded field instances
    (and nu_max with ``with_numax``)."""
    import torch

    feats, ys, nms = [], [], []
    host = dev = None
    for s in seeds:
        if host is None:
            c = workload.Config(cfg.name, cfg.porder, cfg.nx, cfg.jitter, cfg.kind, cfg.nmodes, int(s))
            host = workload.HostCase(c)
            dev = workload.DeviceCase(host, device=device)
        else:
            host = host.with_seed(int(s))
            dev.set_fields(host)
        _, nu, numax = entropy_viscosity(dev)
        f, _ = features(dev)
        ys.append(torch.clamp(nu / torch.clamp(numax, min=1e-30), 0.0, 1.0))
        feats.append(f.clone())
        nms.append(numax.clone())
    if with_numax:
        return torch.cat(feats), torch.cat(ys), torch.cat(nms)
    return torch.cat(feats), torch.cat(ys)


def _event_ms(fn, reps):
    import torch

    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / reps


def _mu_from_nu(dev, nu):
    """mu_e(nelem, ngaus) = rho(node) * nu(element) in the reference's layout."""
    import torch

    n = dev.cfg.nnode
    node = dev.connec.view(n, dev.nelem).long() - 1
    return (dev.rho[node] * nu.view(1, -1)).reshape(-1)


def evaluate(mlp, dev, ybar=None, reps=5):
    """Learned against plain estimator on one field instance: errors, fallback, times.

    ``ybar`` (the training targets' mean y) adds the constant-ratio
    estimator nu = ybar * nu_max, the best feature-free choice in L2."""
    import torch

    from . import kernels

    mu_p, nu_p, numax = entropy_viscosity(dev)
    out_p = [torch.empty_like(x) for x in (dev.Dmass, dev.Dmom, dev.Dener)]
    kernels.full_diffusion_ijk(*dev.geometry(), dev.cfg.Cp, dev.cfg.Pr, dev.rho, dev.u, dev.Tem, dev.mu_fluid, mu_p,
                               dev.mu_sgs, *out_p)
    nu_l, flag = learned_viscosity(mlp, dev)
    out_l = [torch.empty_like(x) for x in out_p]
    diffusion_ijk_nu(dev, nu_l, out_l)

    def rel(a, b):
        return float(torch.linalg.vector_norm((a - b).double()) / max(torch.linalg.vector_norm(b.double()), 1e-300))

    # Two estimators that need no entropy residual, for comparison: the
    # first-order bound nu_max everywhere, and nu_max times the mean training ratio.
    out_b = [torch.empty_like(x) for x in out_p]
    diffusion_ijk_nu(dev, numax, out_b)
    def errs(nu_x, out_x):
        return {"nu_rel_l2": rel(nu_x, nu_p), "Rmass_rel_l2": rel(out_x[0], out_p[0]),
                "Rmom_rel_l2": rel(out_x[1], out_p[1]), "Rener_rel_l2": rel(out_x[2], out_p[2])}

    r = dict(errs(nu_l, out_l))
    r["mu_e_rel_l2"] = rel(_mu_from_nu(dev, nu_l), mu_p)
    r["fallback_fraction"] = float(flag.float().mean())
    r["numax_everywhere"] = errs(numax, out_b)
    if ybar is not None:
        nu_c = float(ybar) * numax
        diffusion_ijk_nu(dev, nu_c, out_b)
        r["constant_ratio"] = errs(nu_c, out_b)
    # The constant fraction of nu_max closest to the plain estimator in the Rmass sense: Rmass is
    # linear in nu, so the best c minimises |c R1 - Rp| with R1 the mass residual of nu_max.
    diffusion_ijk_nu(dev, numax, out_b)
    R1, Rp = out_b[0].double(), out_p[0].double()
    c_best = float(torch.dot(R1, Rp) / torch.clamp(torch.dot(R1, R1), min=1e-300))
    nu_c = c_best * numax
    diffusion_ijk_nu(dev, nu_c, out_b)
    r["best_constant_for_Rmass"] = dict(errs(nu_c, out_b), fraction=c_best)
    diffusion_ijk_nu(dev, torch.zeros_like(numax), out_b)
    r["no_artificial_viscosity"] = errs(torch.zeros_like(numax), out_b)
    mu_buf, nu_buf, nm_buf = torch.empty_like(mu_p), torch.empty_like(nu_p), torch.empty_like(numax)
    nu_lb, flag_b = torch.empty_like(nu_l), torch.empty_like(flag)

    def plain():
        entropy_viscosity(dev, mu_buf, nu_buf, nm_buf)
        kernels.full_diffusion_ijk(*dev.geometry(), dev.cfg.Cp, dev.cfg.Pr, dev.rho, dev.u, dev.Tem, dev.mu_fluid,
                                   mu_buf, dev.mu_sgs, *out_p)

    def learned():
        learned_viscosity(mlp, dev, nu_lb, flag_b)
        diffusion_ijk_nu(dev, nu_lb, out_l)

    r["ms_plain_estimator"] = _event_ms(lambda: entropy_viscosity(dev, mu_buf, nu_buf, nm_buf), reps)
    r["ms_learned_estimator"] = _event_ms(lambda: learned_viscosity(mlp, dev, nu_lb, flag_b), reps)
    r["ms_plain_estimator_plus_diffusion"] = _event_ms(plain, reps)
    r["ms_learned_estimator_plus_diffusion"] = _event_ms(learned, reps)
    # the one-call entry point (the same kernels as learned())
    r["ms_learned_diffusion_call"] = _event_ms(lambda: diffusion_learned(mlp, dev, out_l, nu_lb, flag_b), reps)
    return r


# Feature 0 is log(relative density jump + 1e-12); norm = mean[12], inv_std[12], fmin[12], fmax[12].
_FMAX0 = 3 * NFEAT


def set_trusted_jump(mlp, log_jump_max):
    """Cap the trusted range of feature 0 (the element's relative density jump): elements above
    it take the plain estimator's viscosity (the per-element fallback of both learned paths)."""
    _, norm = mlp.params()
    norm = norm.copy()
    norm[_FMAX0] = min(float(norm[_FMAX0]), float(log_jump_max))
    mlp.set_params(None, norm)


def rmass_error(mlp, dev):
    """Relative L2 of the artificial mass diffusion with the learned viscosity (fallback
    included) against the plain estimator, and the fallback fraction."""
    import torch

    _, nu_p, _ = entropy_viscosity(dev)
    out_p = [torch.empty_like(x) for x in (dev.Dmass, dev.Dmom, dev.Dener)]
    diffusion_ijk_nu(dev, nu_p, out_p)
    nu_l, flag = learned_viscosity(mlp, dev)
    out_l = [torch.empty_like(x) for x in out_p]
    diffusion_ijk_nu(dev, nu_l, out_l)
    d = float(torch.linalg.vector_norm((out_l[0] - out_p[0]).double()))
    return d / max(float(torch.linalg.vector_norm(out_p[0].double())), 1e-300), float(flag.float().mean())


def choose_shock_band(mlp, cfg, feat0, val_seeds, target, fractions=(0.002, 0.005, 0.01, 0.02, 0.03, 0.05, 0.08,
                                                                     0.12, 0.2), device="cuda"):
    """The shock band: the smallest share of elements, by relative density jump (the training
    elements' feature 0 quantiles), whose fallback to the plain estimator brings the artificial
    mass diffusion within ``target`` (relative L2, mean over the validation seeds).  Sets the
    trusted range on the network and returns (log jump threshold, share, validation errors)."""
    import torch

    _, norm0 = mlp.params()
    host = dev = None
    devs = []
    for s in val_seeds:
        c = workload.Config(cfg.name, cfg.porder, cfg.nx, cfg.jitter, cfg.kind, cfg.nmodes, int(s))
        host = workload.HostCase(c) if host is None else host.with_seed(int(s))
        devs.append(host)
    dev = workload.DeviceCase(devs[0], device=device)
    f0 = feat0.double()
    tried = []
    for frac in sorted(fractions):
        thr = float(torch.quantile(f0[torch.randperm(f0.numel(), device=f0.device)[:1 << 22]], 1.0 - frac))
        mlp.set_params(None, norm0)
        set_trusted_jump(mlp, thr)
        errs = []
        for h in devs:
            dev.set_fields(h)
            errs.append(rmass_error(mlp, dev))
        e = float(np.mean([x[0] for x in errs]))
        tried.append({"share": frac, "log_jump_max": thr, "val_Rmass_rel_l2": e,
                      "val_fallback": float(np.mean([x[1] for x in errs]))})
        if e <= target:
            return thr, frac, tried
    return thr, frac, tried


def train_and_evaluate(cfg, train_seeds, eval_seeds, steps=2000, batch=4096, lr=1e-3, seed=0, weights=None,
                       device="cuda", shock_share=0.0, band_target=None, val_seeds=()):
    """Train the network on the plain estimator's output over ``train_seeds``
    and evaluate it on ``eval_seeds`` (the same mesh, other field instances).
    ``shock_share`` > 0 weights the loss towards the shock elements
    (``loss_weights``).  Returns a report dict; writes the weight file if
    ``weights`` is given."""
    import time

    import torch

    t0 = time.time()
    feat, y, nmx = training_data(cfg, train_seeds, device=device, with_numax=True)
    wt = loss_weights(y, nmx, feat, shock_share)
    del nmx
    t_data = time.time() - t0
    mlp = Mlp(seed=seed)
    t0 = time.time()
    loss = mlp.train(feat, y, steps=steps, batch=batch, lr=lr, seed=seed, weight=wt)
    t_train = time.time() - t0
    ybar = float(y.double().mean())
    feat0 = feat.view(-1, NFEAT)[:, 0].clone()
    del feat, y, wt
    torch.cuda.empty_cache()
    band = None
    if band_target is not None:
        thr, share, tried = choose_shock_band(mlp, cfg, feat0, val_seeds, band_target, device=device)
        band = {"target_Rmass_rel_l2": band_target, "val_seeds": [int(s) for s in val_seeds], "log_jump_max": thr,
                "share_of_training_elements": share, "tried": tried}
    del feat0
    if weights:
        mlp.save(weights)
    host = workload.HostCase(workload.Config(cfg.name, cfg.porder, cfg.nx, cfg.jitter, cfg.kind, cfg.nmodes,
                                             int(eval_seeds[0])))
    dev = workload.DeviceCase(host, device=device)
    per_seed = []
    for s in eval_seeds:
        if s != eval_seeds[0]:
            host = host.with_seed(int(s))
            dev.set_fields(host)
        per_seed.append(dict(seed=int(s), **evaluate(mlp, dev, ybar)))

    def mean(key, sub=None):
        v = [(p[sub][key] if sub else p[key]) for p in per_seed]
        return float(np.mean(v))

    keys = ("nu_rel_l2", "mu_e_rel_l2", "Rmass_rel_l2", "Rmom_rel_l2", "Rener_rel_l2", "fallback_fraction",
            "ms_plain_estimator", "ms_learned_estimator", "ms_plain_estimator_plus_diffusion",
            "ms_learned_estimator_plus_diffusion")
    summary = {k: mean(k) for k in keys}
    for sub in ("numax_everywhere", "constant_ratio", "best_constant_for_Rmass", "no_artificial_viscosity"):
        summary[sub] = {k: mean(k, sub) for k in per_seed[0][sub]}
    summary["time_saved_fraction"] = 1.0 - summary["ms_learned_estimator_plus_diffusion"] / \
        summary["ms_plain_estimator_plus_diffusion"]
    return {
        "workload": cfg.name, "porder": cfg.porder, "nelem": cfg.nelem, "npoin": cfg.npoin,
        "train_seeds": [int(s) for s in train_seeds], "eval_seeds": [int(s) for s in eval_seeds],
        "steps": steps, "batch": batch, "lr": lr, "shock_share": shock_share, "shock_band": band,
        "samples": int(len(train_seeds) * cfg.nelem), "ybar": ybar,
        "loss_first_50": float(loss[:50].mean()), "loss_last_50": float(loss[-50:].mean()),
        "seconds_data": t_data, "seconds_train": t_train,
        "mean": summary, "per_seed": per_seed,
    }


def _main(argv=None):
    import argparse
    import json

    ap = argparse.ArgumentParser(description="Train the per-element viscosity network and evaluate it.")
    ap.add_argument("--config", default="learned_48")
    ap.add_argument("--ntrain", type=int, default=64)
    ap.add_argument("--neval", type=int, default=16)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--shock-share", type=float, default=0.0,
                    help="share of the loss weight on the shock elements (see loss_weights)")
    ap.add_argument("--band-target", type=float, default=None,
                    help="Rmass relative L2 the shock-band fallback must reach on the validation seeds")
    ap.add_argument("--nval", type=int, default=2, help="validation seeds (500, 501, ...) for the shock band")
    ap.add_argument("--weights", default=None, help="weight file to write (default data/mlp_<config>.bin)")
    ap.add_argument("--report", default=None, help="report to write (default data/<config>_report.json)")
    a = ap.parse_args(argv)
    cfg = workload.CONFIGS[a.config]
    a.weights = a.weights or shipped_weights(a.config)
    a.report = a.report or os.path.join(DATA, "%s_report.json" % a.config)
    train = list(range(a.ntrain))
    ev = list(range(1000, 1000 + a.neval))
    rep = train_and_evaluate(cfg, train, ev, a.steps, a.batch, a.lr, weights=a.weights, shock_share=a.shock_share,
                             band_target=a.band_target, val_seeds=list(range(500, 500 + a.nval)))
    txt = json.dumps(rep, indent=1)
    if a.report:
        with open(a.report, "w") as f:
            f.write(txt + "\n")
    print(json.dumps(rep["mean"], indent=1))


if __name__ == "__main__":
    _main()
