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

    def train(self, feat, target, steps=2000, batch=4096, lr=1e-3, seed=0, stream=None):
        n = target.numel()
        loss = np.zeros(steps, np.float32)
        capi.call("msod_mlp_train", self.h, _p(feat), _p(target), int(n), int(steps), int(batch), float(lr),
                  int(seed), loss.ctypes.data_as(C.c_void_p), _stream(stream))
        return loss

    def gradient(self, feat, target, idx, stream=None):
        g = np.zeros(NPARAMS, np.float32)
        capi.call("msod_mlp_gradient", self.h, _p(feat), _p(target), _p(idx), int(idx.numel()),
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
