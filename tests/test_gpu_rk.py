"""GPU checks of the lumped mass and the RK4 step (msod_lumped_mass, msod_rk4_step).

Reference: the numpy restatement in the oracle (oracle.lumped_mass, oracle.rk4_step) on the
oracle's FP64 residuals, with the element tables in FP64 and the kernel's own He and gpvol.  The
step is compared through its increments U1 - U0 (the state itself changes little in one step),
within max(1e-4, 3 x floor), the floor being the oracle's own FP32 step (FP32 tables and
residuals) against the FP64 one.
"""
import ctypes as C

import numpy as np
import pytest

from minisod2d_gb300 import capi, timestep, workload
from oracle import oracle as O
from tests import refimpl

pytestmark = pytest.mark.gpu

NAMES = ("rho", "q", "rhoE")


def _case(cuda, P=4, nx=3, kind=0, seed=0, mu=1e-3, Cp=1004.5):
    cfg = workload.Config("rk", P, nx, 0.05, kind, 8, seed, Cp=Cp)
    host = workload.HostCase(cfg)
    rng = np.random.default_rng(seed + 7)
    host.mu_e = (mu * rng.random(host.mu_e.size)).astype(np.float32)
    host.mu_sgs = (0.5 * mu * rng.random(host.mu_sgs.size)).astype(np.float32)
    return host, workload.DeviceCase(host, device=cuda)


def _geom(host, dev, dtype):
    t = O.element_tables(dev.cfg.porder, dtype)
    return dict(t, connec=host.connec, He=dev.He.cpu().numpy().astype(dtype),
                gpvol=dev.gpvol.cpu().numpy().astype(dtype))


def _state(dev):
    return dev.rho.clone(), dev.q.clone(), (dev.rho * dev.E).contiguous()


def test_lumped_mass(cuda):
    host, dev = _case(cuda)
    Ml = timestep.lumped_mass(dev).cpu().numpy()
    ref = O.lumped_mass(dev.cfg.porder, dev.nelem, dev.npoin, host.connec, dev.gpvol.cpu().numpy())
    assert refimpl.rel_l2(Ml, ref) < 1e-6
    assert np.all(Ml > 0)
    assert abs(Ml.astype(np.float64).sum() - 1.0) < 1e-5  # the unit cube


@pytest.mark.parametrize("P,nx,kind", [(4, 3, 0), (5, 2, 1), (2, 4, 0)])
def test_rk4_step_matches_oracle(cuda, P, nx, kind):
    host, dev = _case(cuda, P, nx, kind)
    Ml = timestep.lumped_mass(dev)
    ws = timestep.workspace(dev)
    rho, q, rhoE = _state(dev)
    U0 = [x.cpu().numpy().astype(np.float64) for x in (rho, q, rhoE)]
    dt = 2e-3
    timestep.rk4_step(dev, Ml, dt, rho, q, rhoE, ws)
    got = [x.cpu().numpy().astype(np.float64) for x in (rho, q, rhoE)]
    f = host.fields
    gp = dev.gpvol.cpu().numpy()
    args = (P, dev.nelem, dev.npoin)
    rest = (dev.cfg.Cp, dev.cfg.Pr, timestep.GAMMA, timestep.RGAS)
    ref = O.rk4_step(*args, _geom(host, dev, np.float64), *rest,
                     O.lumped_mass(*args, host.connec, gp, np.float64), f["mu_fluid"], host.mu_e, host.mu_sgs, dt,
                     *U0, dtype=np.float64, nthreads=8)
    ref32 = O.rk4_step(*args, _geom(host, dev, np.float32), *rest,
                       O.lumped_mass(*args, host.connec, gp, np.float32), f["mu_fluid"], host.mu_e, host.mu_sgs,
                       dt, *[u.astype(np.float32) for u in U0], dtype=np.float32, nthreads=8)
    errs = []
    for name, g, r, r32, u0 in zip(NAMES, got, ref, ref32, U0):
        e = refimpl.rel_l2(g - u0, r - u0)
        fl = refimpl.rel_l2(r32.astype(np.float64) - u0, r - u0)
        errs.append((name, e, fl))
    print("RK4 P=%d " % P + " ".join("%s: err %.2e floor %.2e" % x for x in errs))
    for name, e, fl in errs:
        assert e <= max(1e-4, 3.0 * fl), (name, e, fl)


def test_rk4_pure_diffusion_conserves_mass_and_smooths(cuda):
    """u = 0, a uniform pressure, Cp = 0 (no heat flux, so the pressure stays uniform and no flow
    starts) and nu_e = mu_e / rho uniform at the start: only the artificial mass diffusion acts,
    and the density bump spreads.  The reference applies nu_e at the output node, outside the
    weak divergence (elem_diffu.f90:183), so the nodes' mass residuals sum to zero only while nu_e
    is uniform; with mu_e fixed for the step, nu_e drifts as rho changes between stages, and the
    total mass sum(Ml rho) moves at second order: held under 1 % of the mass the diffusion moves."""
    import torch

    cfg = workload.Config("rk", 4, 3, 0.05, 0, 8, 0, Cp=0.0)
    host = workload.HostCase(cfg)
    nu0 = 1e-2
    rho_h = host.fields["rho"]
    host.mu_e = (nu0 * rho_h[host.connec.astype(np.int64) - 1]).astype(np.float32)  # both [a*nelem + e]
    host.mu_sgs = np.zeros_like(host.mu_sgs)
    dev = workload.DeviceCase(host, device=cuda)
    Ml = timestep.lumped_mass(dev)
    ws = timestep.workspace(dev)
    rho = dev.rho.clone()
    q = torch.zeros_like(dev.q)
    rhoE = torch.full_like(dev.rho, 1.0 / (timestep.GAMMA - 1.0))  # p = 1 everywhere
    m0 = float((Ml.double() * rho.double()).sum())
    peak0, low0 = float(rho.max()), float(rho.min())
    for _ in range(3):
        timestep.rk4_step(dev, Ml, 1e-2, rho, q, rhoE, ws)
    m1 = float((Ml.double() * rho.double()).sum())
    moved = float((Ml.double() * (rho.double() - dev.rho.double()).abs()).sum())
    print("RK4 diffusion: mass %.9f -> %.9f (moved %.3e), peak %.6f -> %.6f, low %.6f -> %.6f" % (
        m0, m1, moved, peak0, float(rho.max()), low0, float(rho.min())))
    assert abs(m1 - m0) <= 1e-2 * moved
    assert float(rho.max()) < peak0 and float(rho.min()) > low0


def test_rk4_uniform_state_stays(cuda):
    """A uniform flow is a steady state: every residual vanishes up to the rounding of the tables."""
    import torch

    host, dev = _case(cuda, 4, 3, 0)
    Ml = timestep.lumped_mass(dev)
    ws = timestep.workspace(dev)
    rho = torch.full_like(dev.rho, 1.2)
    u0 = torch.tensor([0.3, -0.1, 0.2], device=cuda)
    q = (1.2 * u0.view(3, 1).expand(3, dev.npoin)).reshape(-1).contiguous()
    rhoE = torch.full_like(dev.rho, 2.5 + 0.5 * 1.2 * float((u0 * u0).sum()))
    r0, q0, e0 = rho.clone(), q.clone(), rhoE.clone()
    timestep.rk4_step(dev, Ml, 1e-2, rho, q, rhoE, ws)
    for a, b in ((rho, r0), (q, q0), (rhoE, e0)):
        assert float((a - b).abs().max()) <= 1e-6 * float(b.abs().max())


def test_rk4_rejects_bad_arguments(cuda):
    host, dev = _case(cuda)
    Ml = timestep.lumped_mass(dev)
    ws = timestep.workspace(dev)
    rho, q, rhoE = _state(dev)
    with pytest.raises(capi.MsodError) as ei:
        timestep.rk4_step(dev, Ml, 1e-3, rho, q, rhoE, ws[: ws.numel() // 2])
    assert ei.value.code == capi.MSOD_ERR_INVALID_ARG
    with pytest.raises(capi.MsodError) as ei:
        timestep.rk4_step(dev, Ml, float("nan"), rho, q, rhoE, ws)
    assert ei.value.code == capi.MSOD_ERR_INVALID_ARG
    with pytest.raises(capi.MsodError) as ei:  # a workspace that does not start on a float boundary
        timestep.rk4_step(dev, Ml, 1e-3, rho, q, rhoE, ws[1:])
    assert ei.value.code == capi.MSOD_ERR_INVALID_ARG
    n = C.c_size_t(0)
    assert capi.lib().msod_rk4_workspace_bytes(dev.npoin, C.byref(n)) == capi.MSOD_OK
    assert n.value == 26 * 4 * dev.npoin


def test_rk4_step_follows_the_mode(cuda):
    """The stages call msod_convec_diffusion_ijk, which makes the two drop-in calls while a form
    other than the default is selected, so the form msod_set_mode selects applies:
    with the FP16 tensor-core kernels the step's increments agree with the FP32 step's to the
    mixed kernels' accuracy, and differ from them (the other kernels ran)."""
    from minisod2d_gb300 import kernels

    host, dev = _case(cuda, 4, 3, 0)
    Ml = timestep.lumped_mass(dev)
    ws = timestep.workspace(dev)
    r32, q32, e32 = _state(dev)
    U0 = [x.clone() for x in (r32, q32, e32)]
    timestep.rk4_step(dev, Ml, 2e-3, r32, q32, e32, ws)
    r16, q16, e16 = (x.clone() for x in U0)
    kernels.set_mode("fp16")
    try:
        timestep.rk4_step(dev, Ml, 2e-3, r16, q16, e16, ws)
    finally:
        kernels.set_mode("fp32")
    for name, a, b, u0 in zip(NAMES, (r16, q16, e16), (r32, q32, e32), U0):
        da, db = (a - u0).double().cpu().numpy(), (b - u0).double().cpu().numpy()
        e = refimpl.rel_l2(da, db)
        print("RK4 fp16 vs fp32 %s: %.2e" % (name, e))
        assert 0.0 < e < 1e-4, (name, e)


def test_rk4_step_captured_in_a_cuda_graph(cuda):
    """The step issues only capturable stream work (device copies, the residual calls' memsets and
    kernels, the stage kernels): two replays of a captured step equal two eager steps."""
    import torch

    host, dev = _case(cuda, 4, 3, 0)
    Ml = timestep.lumped_mass(dev)
    ws = timestep.workspace(dev)
    rho, q, rhoE = _state(dev)
    U0 = [x.clone() for x in (rho, q, rhoE)]
    for _ in range(2):
        timestep.rk4_step(dev, Ml, 2e-3, rho, q, rhoE, ws)
    eager = [x.clone() for x in (rho, q, rhoE)]
    for x, x0 in zip((rho, q, rhoE), U0):
        x.copy_(x0)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(device=cuda)
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            timestep.rk4_step(dev, Ml, 2e-3, rho, q, rhoE, ws, stream=side.cuda_stream)
    for x, x0 in zip((rho, q, rhoE), U0):  # the capture ran nothing; start again from U0
        x.copy_(x0)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip((rho, q, rhoE), eager):
        assert refimpl.rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 1e-6
