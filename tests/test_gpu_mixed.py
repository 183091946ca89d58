"""GPU checks of the mixed-precision convection (FP16 / BF16 hi + lo tensor-core
contractions, FP64 scatter and energy-flux assembly).

Reference: the FP64 oracle with the element tables in FP64 (as the
reference's FP64 build computes them) and the FP32 fields, He and gpvol the
kernel reads, promoted to FP64.  The plain FP32 GPU kernel's distance from the
same FP64 answer (the FP32 floor) is printed beside each result.
Criteria per residual (relative L2):
  * convection: <= 1e-4 for both formats and <= 1e-5 for FP16;
  * diffusion: <= 1e-4 for FP16 and <= max(5e-4, 6 x floor) for BF16.  The
    weak divergence cancels strongly between neighbouring elements, which
    magnifies the FP32 rounding of the derivative tables acting on the fields'
    means in the plain kernel (its floor reaches 2e-3 for the energy residual
    of the 32^3 porder-7 workload); the mixed kernels contract the fields minus
    their value at one node of the element, so the rounded tables act on the
    variation only, and FP16 stays within 1e-4; the BF16 splits (2 x 8
    significant bits) reach 2-4e-4 on these small cases.
"""
import numpy as np
import pytest

from minisod2d_gb300 import workload
from oracle import oracle as O
from tests import refimpl

pytestmark = pytest.mark.gpu

TOL = 1e-4
TOL_FP16 = 1e-5
DIFFU_FLOOR_FACTOR = 6.0
BF16_DIFFU_TOL = 5e-4


def _case(cuda, P, nx, kind=0, nmodes=8, seed=0, jitter=0.05):
    cfg = workload.Config("t", P, nx, jitter, kind, nmodes, seed)
    host = workload.HostCase(cfg)
    return host, workload.DeviceCase(host, device=cuda)


def _geom64(host, dev):
    """FP64 element tables (the reference's FP64 build) with the kernel's own He and gpvol."""
    t64 = O.element_tables(dev.cfg.porder, np.float64)
    return dict(t64, connec=host.connec, He=dev.He.cpu().numpy().astype(np.float64),
                gpvol=dev.gpvol.cpu().numpy().astype(np.float64))


def _oracle64(host, dev):
    geom = _geom64(host, dev)
    f = host.fields
    return O.full_convec_ijk(dev.cfg.porder, dev.nelem, dev.npoin, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"],
                             dtype=np.float64, nthreads=8)


def _errs(gpu, ref):
    return [refimpl.rel_l2(g.cpu().numpy().astype(np.float64), r) for g, r in zip(gpu, ref)]


@pytest.mark.parametrize("P,nx,kind,nmodes", [(7, 3, 0, 16), (5, 4, 1, 8), (4, 4, 0, 8), (2, 5, 1, 8)])
def test_mixed_convection_vs_fp64_oracle(cuda, P, nx, kind, nmodes):
    host, dev = _case(cuda, P, nx, kind, nmodes)
    ref = _oracle64(host, dev)
    floor = _errs(dev.convec(), ref)
    for prec in ("fp16", "bf16"):
        errs = _errs(dev.convec_mixed(prec), ref)
        print("MIXED P=%d kind=%d %s err=%s floor32=%s" % (
            P, kind, prec, ["%.2e" % x for x in errs], ["%.2e" % x for x in floor]))
        for name, e, fl in zip(("mass", "mom", "ener"), errs, floor):
            assert e <= TOL, (prec, name, e)
            if prec == "fp16":
                assert e <= TOL_FP16, (prec, name, e, fl)


def test_mixed_convection_deterministic_inputs_and_intent_out(cuda):
    import torch

    host, dev = _case(cuda, 7, 2, 0, 16, seed=3)
    a = dev.convec_mixed("fp16")
    out = tuple(torch.full_like(x, 7.0) for x in a)
    b = dev.convec_mixed("fp16", out=out)
    for x, y in zip(a, b):
        # atomics reorder the per-node sums; values agree to rounding
        assert refimpl.rel_l2(x.cpu().numpy(), y.cpu().numpy()) < 1e-12


def test_mixed_convection_constant_fields_give_zero(cuda):
    """Constant fields: every derivative vanishes exactly (the shift by the
    reference node makes the split inputs exactly zero)."""
    import torch

    host, dev = _case(cuda, 5, 3, 0, 8)
    for t, v in ((dev.rho, 1.25), (dev.pr, 0.8), (dev.E, 2.5)):
        t.fill_(v)
    dev.u.fill_(0.3)
    dev.q.fill_(0.375)
    for prec in ("fp16", "bf16"):
        for x in dev.convec_mixed(prec):
            assert float(torch.abs(x).max()) == 0.0


def test_mixed_rejects_bad_arguments(cuda):
    import torch

    from minisod2d_gb300 import capi, kernels

    host, dev = _case(cuda, 4, 2)
    out = dev.convec_mixed("fp16")
    g = dev.geometry()
    args = [g[0], g[1], g[2], g[5], g[6], g[7], *g[9:], dev.u, dev.q, dev.rho, dev.pr, dev.E]
    with pytest.raises(TypeError):
        kernels.full_convec_ijk_mixed(*args, dev.Rmass, dev.Rmom, dev.Rener)  # FP32 outputs
    with pytest.raises(capi.MsodError) as ei:
        capi.call("msod_convec_ijk_mixed", 5, 4, dev.nelem, dev.npoin, *[t.data_ptr() for t in args[2:]],
                  *[t.data_ptr() for t in out], torch.cuda.current_stream().cuda_stream)
    assert ei.value.code == capi.MSOD_ERR_INVALID_ARG


def _diffu_case(cuda, P, nx, kind, nmodes, mu=1e-3, seed=0):
    cfg = workload.Config("t", P, nx, 0.05, kind, nmodes, seed)
    host = workload.HostCase(cfg)
    rng = np.random.default_rng(seed + 11)
    host.mu_e = (mu * rng.random(host.mu_e.size)).astype(np.float32)
    host.mu_sgs = (0.5 * mu * rng.random(host.mu_sgs.size)).astype(np.float32)
    return host, workload.DeviceCase(host, device=cuda)


def _diffu_oracle64(host, dev, mu_e=None):
    geom = _geom64(host, dev)
    f = host.fields
    return O.full_diffusion_ijk(dev.cfg.porder, dev.nelem, dev.npoin, geom, dev.cfg.Cp, dev.cfg.Pr, f["rho"], f["u"],
                                f["Tem"], f["mu_fluid"], host.mu_e if mu_e is None else mu_e, host.mu_sgs,
                                dtype=np.float64, nthreads=8)


@pytest.mark.parametrize("P,nx,kind,nmodes", [(7, 3, 0, 16), (5, 4, 1, 8), (4, 4, 0, 8), (2, 5, 1, 8)])
def test_mixed_diffusion_vs_fp64_oracle(cuda, P, nx, kind, nmodes):
    host, dev = _diffu_case(cuda, P, nx, kind, nmodes)
    ref = _diffu_oracle64(host, dev)
    floor = _errs(dev.diffu(), ref)
    for prec in ("fp16", "bf16"):
        errs = _errs(dev.diffu_mixed(prec), ref)
        print("MIXED-DIFFU P=%d kind=%d %s err=%s floor32=%s" % (
            P, kind, prec, ["%.2e" % x for x in errs], ["%.2e" % x for x in floor]))
        for name, e, fl in zip(("mass", "mom", "ener"), errs, floor):
            bound = TOL if prec == "fp16" else max(BF16_DIFFU_TOL, DIFFU_FLOOR_FACTOR * fl)
            assert e <= bound, (prec, name, e, fl)


def test_mixed_diffusion_per_element_viscosity(cuda):
    """The _nu form equals the mu_e-array form with mu_e(e, a) = rho(a) nu(e)."""
    import torch

    host, dev = _diffu_case(cuda, 5, 3, 1, 8)
    nu = torch.rand(dev.nelem, device=cuda) * 1e-3
    n = dev.cfg.nnode
    node = dev.connec.view(n, dev.nelem).long() - 1
    mu_arr = (dev.rho[node] * nu.view(1, -1)).reshape(-1).contiguous()
    a = dev.diffu_mixed("fp16", nu_elem=nu)
    b = dev.diffu_mixed("fp16", mu_e=mu_arr)
    for x, y in zip(a, b):
        assert refimpl.rel_l2(x.cpu().numpy(), y.cpu().numpy()) < 1e-6
