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
    """Diffusion with the network evaluated in the diffusion kernel's prologue
    (features from rho, u and the pressure, or p = rho Rgas T with ``from_T``;
    plain-estimator fallback per element).  Returns the residuals, the
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


def training_data(cfg, seeds, device="cuda"):
    """Features and targets y = nu / nu_max of the plain estimator over seeded field instances."""
    import torch

    feats, ys = [], []
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
    r = {
        "nu_rel_l2": rel(nu_l, nu_p),
        "mu_e_rel_l2": rel(_mu_from_nu(dev, nu_l), mu_p),
        "Rmass_rel_l2": rel(out_l[0], out_p[0]),
        "Rmom_rel_l2": rel(out_l[1], out_p[1]),
        "Rener_rel_l2": rel(out_l[2], out_p[2]),
        "fallback_fraction": float(flag.float().mean()),
        "numax_everywhere": {"nu_rel_l2": rel(numax, nu_p), "Rmom_rel_l2": rel(out_b[1], out_p[1]),
                             "Rener_rel_l2": rel(out_b[2], out_p[2])},
    }
    if ybar is not None:
        nu_c = float(ybar) * numax
        diffusion_ijk_nu(dev, nu_c, out_b)
        r["constant_ratio"] = {"nu_rel_l2": rel(nu_c, nu_p), "Rmom_rel_l2": rel(out_b[1], out_p[1]),
                               "Rener_rel_l2": rel(out_b[2], out_p[2])}
    diffusion_ijk_nu(dev, torch.zeros_like(numax), out_b)
    r["no_artificial_viscosity"] = {"nu_rel_l2": 1.0, "Rmom_rel_l2": rel(out_b[1], out_p[1]),
                                    "Rener_rel_l2": rel(out_b[2], out_p[2])}
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
    # the network evaluated in the diffusion prologue (features + fallback + fused diffusion)
    r["ms_fused_learned_diffusion"] = _event_ms(lambda: diffusion_learned(mlp, dev, out_l, nu_lb, flag_b), reps)
    return r


def train_and_evaluate(cfg, train_seeds, eval_seeds, steps=2000, batch=4096, lr=1e-3, seed=0, weights=None,
                       device="cuda"):
    """Train the network on the plain estimator's output over ``train_seeds``
    and evaluate it on ``eval_seeds`` (the same mesh, other field instances).
    Returns a report dict; writes the weight file if ``weights`` is given."""
    import time

    import torch

    t0 = time.time()
    feat, y = training_data(cfg, train_seeds, device=device)
    t_data = time.time() - t0
    mlp = Mlp(seed=seed)
    t0 = time.time()
    loss = mlp.train(feat, y, steps=steps, batch=batch, lr=lr, seed=seed)
    t_train = time.time() - t0
    ybar = float(y.double().mean())
    del feat, y
    torch.cuda.empty_cache()
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
    for sub in ("numax_everywhere", "constant_ratio", "no_artificial_viscosity"):
        summary[sub] = {k: mean(k, sub) for k in per_seed[0][sub]}
    summary["time_saved_fraction"] = 1.0 - summary["ms_learned_estimator_plus_diffusion"] / \
        summary["ms_plain_estimator_plus_diffusion"]
    return {
        "workload": cfg.name, "porder": cfg.porder, "nelem": cfg.nelem, "npoin": cfg.npoin,
        "train_seeds": [int(s) for s in train_seeds], "eval_seeds": [int(s) for s in eval_seeds],
        "steps": steps, "batch": batch, "lr": lr, "samples": int(len(train_seeds) * cfg.nelem), "ybar": ybar,
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
    ap.add_argument("--weights", default=None, help="weight file to write (default data/mlp_<config>.bin)")
    ap.add_argument("--report", default=None, help="report to write (default data/<config>_report.json)")
    a = ap.parse_args(argv)
    cfg = workload.CONFIGS[a.config]
    a.weights = a.weights or shipped_weights(a.config)
    a.report = a.report or os.path.join(DATA, "%s_report.json" % a.config)
    train = list(range(a.ntrain))
    ev = list(range(1000, 1000 + a.neval))
    rep = train_and_evaluate(cfg, train, ev, a.steps, a.batch, a.lr, weights=a.weights)
    txt = json.dumps(rep, indent=1)
    if a.report:
        with open(a.report, "w") as f:
            f.write(txt + "\n")
    print(json.dumps(rep["mean"], indent=1))


if __name__ == "__main__":
    _main()
