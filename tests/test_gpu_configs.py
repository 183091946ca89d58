"""GPU parity at the mixed-precision (32^3 porder 7) and combined (96^3 porder 5) workloads.

Both workloads are run whole on the GPU; a slab of element layers from the middle of the mesh is
run again through the C ABI and by the FP32 / FP64 oracles, and compared on the slab's fully
assembled nodes (every element around them lies in the slab), as tests/test_gpu_parity.py does for
the 64^3 porder-4 workload.  Criteria (relative L2 per residual):
  * plain FP32 kernels: the module criterion of tests/test_gpu_parity.py (1e-5 against the FP32
    oracle, or within the FP32 floor where that floor exceeds 1e-5);
  * mixed-precision kernels against the FP64 oracle: convection <= 1e-4 (FP16 and BF16);
    diffusion <= 1e-4 (FP16) and <= 3e-3 (BF16).  The BF16 splits carry 2 x 8 significant bits,
    and the weak divergence, which cancels between neighbouring elements, magnifies their error:
    measured 2.2e-3 (momentum) and 2.4e-3 (energy) at 32^3 porder 7, where FP16 gives 3.4e-5 and
    3.2e-5 and the FP32 kernels 7.5e-5 and 2.4e-3 (the FP64 energy assembly of the mixed kernels
    avoids the FP32 cancellation of the energy residual);
  * viscosity from the estimators (96^3 porder 5): the diffusion kernel with the per-element
    viscosity of the plain estimator and of the shipped network, each against the oracle with the
    same mu_e(e, a) = rho(a) nu(e).
"""
import ctypes as C

import numpy as np
import pytest

from minisod2d_gb300 import capi, kernels, learn, workload
from oracle import oracle as O
from tests import refimpl
from tests.test_gpu_parity import NTH, TOL32, _compare, _geom64

pytestmark = pytest.mark.gpu


def _cpu(x):
    return x.cpu().numpy()


class Slab:
    """`layers` element layers (z) from the middle of a structured nx^3 mesh on the device."""

    def __init__(self, host, dev, layers, cuda):
        import torch

        n, P, nx = host.cfg.nnode, host.cfg.porder, host.cfg.nx
        z0 = nx // 2 - layers // 2
        z1 = z0 + layers
        self.e0, self.e1 = z0 * nx * nx, z1 * nx * nx
        NX = nx * P + 1
        K = np.arange(host.npoin) // (NX * NX)
        self.inner = (K > z0 * P) & (K < z1 * P)
        self.ne = self.e1 - self.e0
        e0, e1 = self.e0, self.e1
        self.con = np.ascontiguousarray(host.connec.reshape(n, host.nelem)[:, e0:e1]).reshape(-1)
        He = _cpu(dev.He).reshape(host.nelem, -1)[e0:e1].reshape(-1)
        gp = _cpu(dev.gpvol).reshape(host.nelem, -1)[e0:e1].reshape(-1)
        self.geom = dict(host.tables, connec=self.con, He=He, gpvol=gp)
        self.g64 = _geom64(self.geom)
        self.d_con, self.d_He, self.d_gp = (torch.from_numpy(x).to(cuda) for x in (self.con, He, gp))
        self.geo = (self.ne, dev.npoin, self.d_con, None, None, self.d_He, self.d_gp, dev.dlxigp_ip, None,
                    dev.invAtoIJK, dev.AtoI, dev.AtoJ, dev.AtoK)
        self.P, self.n, self.npoin = P, n, dev.npoin

    def mask(self, x):
        return [np.asarray(v)[np.tile(self.inner, len(np.asarray(v)) // len(self.inner))] for v in x]

    def elem_array(self, a):
        """The slab's part of an array in the mu_e(nelem, ngaus) layout (a[g*nelem + e])."""
        a = np.asarray(a).reshape(self.n, -1)
        return np.ascontiguousarray(a[:, self.e0:self.e1]).reshape(-1)

    def oracle_convec(self, f, dtype=np.float32):
        g = self.geom if dtype == np.float32 else self.g64
        return O.full_convec_ijk(self.P, self.ne, self.npoin, g, f["u"], f["q"], f["rho"], f["pr"], f["E"], dtype,
                                 nthreads=NTH)

    def oracle_diffu(self, cfg, f, mu_e, mu_sgs, dtype=np.float32):
        g = self.geom if dtype == np.float32 else self.g64
        return O.full_diffusion_ijk(self.P, self.ne, self.npoin, g, cfg.Cp, cfg.Pr, f["rho"], f["u"], f["Tem"],
                                    f["mu_fluid"], mu_e, mu_sgs, dtype, nthreads=NTH)


def _out64(dev):
    import torch

    return tuple(torch.empty(k * dev.npoin, dtype=torch.float64, device=dev.He.device) for k in (1, 3, 1))


def _mixed_check(label, got, ref64, floors, diffusion, prec):
    errs = [refimpl.rel_l2(g, r) for g, r in zip(got, ref64)]
    print("CONFIG %s %s err=%s floor32=%s" % (label, prec, ["%.2e" % e for e in errs], ["%.2e" % f for f in floors]))
    for name, e, fl in zip(("mass", "mom", "ener"), errs, floors):
        if np.isnan(e):
            continue
        bound = (1e-4 if prec == "fp16" else 3e-3) if diffusion else 1e-4
        assert e <= bound, (label, prec, name, e, fl)
    return errs


def test_sampled_parity_mixed_p7(cuda):
    """32^3 hexes, porder 7, jittered, 16-mode fields: plain FP32 kernels against the oracle and
    the FP16 / BF16 tensor-core kernels against the FP64 oracle, on a two-layer slab."""
    import torch

    cfg = workload.CONFIGS["mixed_p7"]
    host = workload.HostCase(cfg)
    dev = workload.DeviceCase(host, device=cuda)
    s = Slab(host, dev, 2, cuda)
    f = host.fields
    kernels.full_convec_ijk(*s.geo, dev.u, dev.q, dev.rho, dev.pr, dev.E, dev.Rmass, dev.Rmom, dev.Rener)
    r32, r64 = s.oracle_convec(f), s.oracle_convec(f, np.float64)
    got = [_cpu(x) for x in (dev.Rmass, dev.Rmom, dev.Rener)]
    cerr = _compare(s.mask(got), s.mask(r32), TOL32, "convec mixed_p7 slab", s.mask(r64))
    mu = np.zeros(s.ne * s.n, np.float32)
    d_mu = torch.from_numpy(mu).to(cuda)
    kernels.full_diffusion_ijk(*s.geo, cfg.Cp, cfg.Pr, dev.rho, dev.u, dev.Tem, dev.mu_fluid, d_mu, d_mu, dev.Dmass,
                               dev.Dmom, dev.Dener)
    d32, d64 = s.oracle_diffu(cfg, f, mu, mu), s.oracle_diffu(cfg, f, mu, mu, np.float64)
    got = [_cpu(x) for x in (dev.Dmass, dev.Dmom, dev.Dener)]
    derr = _compare(s.mask(got), s.mask(d32), TOL32, "diffu mixed_p7 slab", s.mask(d64))
    out = _out64(dev)
    geo_m = (s.ne, dev.npoin, s.d_con, s.d_He, s.d_gp, dev.dlxigp_ip, dev.invAtoIJK, dev.AtoI, dev.AtoJ, dev.AtoK)
    for prec in ("fp16", "bf16"):
        kernels.full_convec_ijk_mixed(*geo_m, dev.u, dev.q, dev.rho, dev.pr, dev.E, *out, precision=prec)
        _mixed_check("convec mixed_p7 slab", s.mask([_cpu(x) for x in out]), s.mask(r64), [e[1] for e in cerr],
                     False, prec)
        kernels.full_diffusion_ijk_mixed(*geo_m, cfg.Cp, cfg.Pr, dev.rho, dev.u, dev.Tem, dev.mu_fluid, d_mu, d_mu,
                                         *out, precision=prec)
        _mixed_check("diffu mixed_p7 slab", s.mask([_cpu(x) for x in out]), s.mask(d64), [e[1] for e in derr],
                     True, prec)


def test_sampled_parity_combined_96(cuda):
    """96^3 hexes, porder 5, jittered, shock-like fields (the combined workload): on a two-layer
    slab, the plain FP32 convection; the diffusion with the plain estimator's viscosity and with
    the shipped network's (both estimated on the whole mesh), each against the oracles with the
    same mu_e; and the mixed FP16 diffusion with the network's viscosity against the FP64 oracle."""
    import torch

    cfg = workload.CONFIGS["combined_96"]
    host = workload.HostCase(workload.Config(cfg.name, cfg.porder, cfg.nx, cfg.jitter, cfg.kind, cfg.nmodes, 2024))
    dev = workload.DeviceCase(host, device=cuda)
    s = Slab(host, dev, 2, cuda)
    f = host.fields
    kernels.full_convec_ijk(*s.geo, dev.u, dev.q, dev.rho, dev.pr, dev.E, dev.Rmass, dev.Rmom, dev.Rener)
    r32, r64 = s.oracle_convec(f), s.oracle_convec(f, np.float64)
    got = [_cpu(x) for x in (dev.Rmass, dev.Rmom, dev.Rener)]
    _compare(s.mask(got), s.mask(r32), TOL32, "convec combined_96 slab", s.mask(r64))
    # viscosities on the whole mesh: the plain estimator and the shipped network
    _, nu_p, _ = learn.entropy_viscosity(dev)
    m = learn.Mlp()
    m.load(learn.shipped_weights("combined_96"))
    nu_l, flag = learn.learned_viscosity(m, dev)
    n = s.n
    node = s.con.reshape(n, s.ne) - 1
    out = (dev.Dmass, dev.Dmom, dev.Dener)
    mu_sgs = s.elem_array(host.mu_sgs)
    d_sgs = torch.from_numpy(mu_sgs).to(cuda)
    for label, nu in (("plain estimator", nu_p), ("network", nu_l)):
        nu_s = nu[s.e0:s.e1].contiguous()
        g = s.geo
        capi.call("msod_diffusion_ijk_nu", s.P, g[0], g[1], C.c_void_p(g[2].data_ptr()), C.c_void_p(g[5].data_ptr()),
                  C.c_void_p(g[6].data_ptr()), C.c_void_p(g[7].data_ptr()), C.c_void_p(g[9].data_ptr()),
                  C.c_void_p(g[10].data_ptr()), C.c_void_p(g[11].data_ptr()), C.c_void_p(g[12].data_ptr()),
                  C.c_float(cfg.Cp), C.c_float(cfg.Pr), C.c_void_p(dev.rho.data_ptr()), C.c_void_p(dev.u.data_ptr()),
                  C.c_void_p(dev.Tem.data_ptr()), C.c_void_p(dev.mu_fluid.data_ptr()), C.c_void_p(nu_s.data_ptr()),
                  C.c_void_p(d_sgs.data_ptr()), *[C.c_void_p(o.data_ptr()) for o in out],
                  torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        # the oracle's mu_e(e, a) = rho(a) nu(e), rounded as the kernel rounds it
        mu = (f["rho"][node] * _cpu(nu_s)[None, :]).astype(np.float32).reshape(-1)
        d32, d64 = s.oracle_diffu(cfg, f, mu, mu_sgs), s.oracle_diffu(cfg, f, mu, mu_sgs, np.float64)
        got = [_cpu(x) for x in out]
        derr = _compare(s.mask(got), s.mask(d32), TOL32, "diffu combined_96 slab (%s)" % label, s.mask(d64))
    # the mixed FP16 diffusion with the network's viscosity (the workload's full form)
    o64 = _out64(dev)
    geo_m = (s.ne, dev.npoin, s.d_con, s.d_He, s.d_gp, dev.dlxigp_ip, dev.invAtoIJK, dev.AtoI, dev.AtoJ, dev.AtoK)
    kernels.full_diffusion_ijk_mixed(*geo_m, cfg.Cp, cfg.Pr, dev.rho, dev.u, dev.Tem, dev.mu_fluid, None, d_sgs, *o64,
                                     precision="fp16", nu_elem=nu_l[s.e0:s.e1].contiguous())
    _mixed_check("diffu combined_96 slab (network, fp16)", s.mask([_cpu(x) for x in o64]), s.mask(d64),
                 [e[1] for e in derr], True, "fp16")
    print("CONFIG combined_96 fallback fraction %.2e" % float(flag.float().mean()))
