"""GPU parity of the plain kernels against the CPU oracle, through the C ABI.

Tolerance: relative L2 <= 1e-5 per residual in FP32 (atomic scatter order and
the kernels' re-associated sums differ from the reference's Fortran order);
<= 1e-11 for the FP64 builds.  Connectivity and index handling are exact by
construction (the kernels read the caller's connec / invAtoIJK / gmshAtoI/J/K).
"""
import os

import numpy as np
import pytest

from minisod2d_gb300 import capi, fem, kernels, workload
from oracle import oracle as O
from tests import refimpl

pytestmark = pytest.mark.gpu

TOL32 = 1e-5
TOL64 = 1e-11
NTH = max(1, min(16, os.cpu_count() or 1))


def _case(cuda, P, nx, jitter=0.05, kind=0, seed=0, mu=0.0, dtype=None):
    import torch

    cfg = workload.Config("t", P, nx, jitter, kind, 8, seed)
    host = workload.HostCase(cfg)
    if mu:
        rng = np.random.default_rng(seed + 11)
        host.mu_e = (mu * rng.random(host.mu_e.size)).astype(np.float32)
        host.mu_sgs = (0.5 * mu * rng.random(host.mu_sgs.size)).astype(np.float32)
    dev = workload.DeviceCase(host, device=cuda, dtype=dtype or torch.float32)
    return host, dev


def _geom_host(dev):
    t = dev.host.tables
    return dict(t, connec=dev.host.connec, He=dev.He.cpu().numpy(), gpvol=dev.gpvol.cpu().numpy())


def _cpu(x):
    return x.cpu().numpy()


def _compare(gpu, ref, tol, label):
    errs = []
    for name, g, r in zip(("mass", "mom", "ener"), gpu, ref):
        g = _cpu(g) if not isinstance(g, np.ndarray) else g
        if np.linalg.norm(r) == 0.0:
            assert np.abs(g).max() == 0.0, (label, name)
            errs.append(0.0)
            continue
        e = refimpl.rel_l2(g, r)
        errs.append(e)
        assert e <= tol, (label, name, e)
    print("PARITY %s rel_l2 mass=%.3e mom=%.3e ener=%.3e" % (label, *errs))
    return errs


def _oracle_convec(host, geom, dtype=np.float32):
    f = host.fields
    return O.full_convec_ijk(host.cfg.porder, host.nelem, host.npoin, geom, f["u"], f["q"], f["rho"], f["pr"],
                             f["E"], dtype, nthreads=NTH)


def _oracle_diffu(host, geom, dtype=np.float32):
    f = host.fields
    c = host.cfg
    return O.full_diffusion_ijk(c.porder, host.nelem, host.npoin, geom, c.Cp, c.Pr, f["rho"], f["u"], f["Tem"],
                                f["mu_fluid"], host.mu_e, host.mu_sgs, dtype, nthreads=NTH)


@pytest.mark.parametrize("P,nx", [(4, 4), (7, 2), (2, 3)])
def test_jacobian_bit_exact(cuda, P, nx):
    host, dev = _case(cuda, P, nx, jitter=0.05)
    t = host.tables
    He, gp = O.elem_jacobian(P, host.nelem, host.npoin, host.connec, host.coord, t["dNgp"], t["wgp"], np.float32)
    assert np.array_equal(_cpu(dev.He).view(np.uint32), He.view(np.uint32))
    assert np.array_equal(_cpu(dev.gpvol).view(np.uint32), gp.view(np.uint32))


def test_convec_parity_plain_16(cuda):
    """The CPU-runnable workload: 16^3 hexes, porder 4, affine mesh, smooth fields."""
    host, dev = _case(cuda, 4, 16, jitter=0.0)
    g = dev.convec()
    r = _oracle_convec(host, _geom_host(dev))
    _compare(g, r, TOL32, "convec plain_16")


def test_diffu_parity_plain_16(cuda):
    host, dev = _case(cuda, 4, 16, jitter=0.0)
    g = dev.diffu()
    r = _oracle_diffu(host, _geom_host(dev))
    _compare(g, r, TOL32, "diffu plain_16")


@pytest.mark.parametrize("P", range(1, 9))
def test_parity_all_porders(cuda, P):
    nx = 3 if P <= 4 else 2
    host, dev = _case(cuda, P, nx, jitter=0.05, kind=P % 2, seed=P, mu=2e-3)
    geom = _geom_host(dev)
    _compare(dev.convec(), _oracle_convec(host, geom), TOL32, "convec P=%d" % P)
    _compare(dev.diffu(), _oracle_diffu(host, geom), TOL32, "diffu P=%d" % P)


@pytest.mark.parametrize("P", [2, 4, 7])
def test_parity_fp64(cuda, P):
    import torch

    host, dev = _case(cuda, P, 2, jitter=0.05, kind=1, seed=3, mu=2e-3, dtype=torch.float64)
    geom = dict(O.element_tables(P, np.float64), connec=host.connec, He=_cpu(dev.He), gpvol=_cpu(dev.gpvol))
    f64 = {k: v.astype(np.float64) for k, v in host.fields.items()}
    r = O.full_convec_ijk(P, host.nelem, host.npoin, geom, f64["u"], f64["q"], f64["rho"], f64["pr"], f64["E"],
                          np.float64, nthreads=NTH)
    _compare(dev.convec(), r, TOL64, "convec f64 P=%d" % P)
    r = O.full_diffusion_ijk(P, host.nelem, host.npoin, geom, host.cfg.Cp, host.cfg.Pr, f64["rho"], f64["u"],
                             f64["Tem"], f64["mu_fluid"], host.mu_e.astype(np.float64),
                             host.mu_sgs.astype(np.float64), np.float64, nthreads=NTH)
    _compare(dev.diffu(), r, TOL64, "diffu f64 P=%d" % P)


def test_reference_driver_case(cuda):
    """The reference driver's own case (main.f90:320-413): disconnected mesh,
    nodes 1 and 4 of each element perturbed, mu = 1, Cp = Pr = 1."""
    import torch

    P, ne = 4, 7
    t = O.element_tables(P)
    connec, coord = O.create_mesh_disconnected(P, ne, t["xgp"])
    npn = ne * t["n"]
    He, gp = O.elem_jacobian(P, ne, npn, connec, coord, t["dNgp"], t["wgp"])
    f = O.reference_ic(P, ne, npn, connec)
    geom = dict(t, connec=connec, He=He, gpvol=gp)
    d = {k: torch.from_numpy(v).to(cuda) for k, v in dict(geom, **f).items() if isinstance(v, np.ndarray)}
    out = [torch.empty(npn, device=cuda), torch.empty(3 * npn, device=cuda), torch.empty(npn, device=cuda)]
    geo = (ne, npn, d["connec"], None, None, d["He"], d["gpvol"], d["dlxigp_ip"], None, d["invAtoIJK"], d["AtoI"],
           d["AtoJ"], d["AtoK"])
    kernels.full_convec_ijk(*geo, d["u"], d["q"], d["rho"], d["pr"], d["E"], *out)
    r = O.full_convec_ijk(P, ne, npn, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"])
    _compare(out, r, TOL32, "convec reference-driver case")
    kernels.full_convec_ijk_split(*geo, d["u"], d["q"], d["rho"], d["pr"], d["E"], *out)
    r = O.full_convec_ijk(P, ne, npn, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], split=True)
    _compare(out, r, TOL32, "convec_split reference-driver case")
    kernels.full_diffusion_ijk(*geo, 1.0, 1.0, d["rho"], d["u"], d["Tem"], d["mu_fluid"], d["mu_e"], d["mu_sgs"], *out)
    r = O.full_diffusion_ijk(P, ne, npn, geom, 1.0, 1.0, f["rho"], f["u"], f["Tem"], f["mu_fluid"], f["mu_e"],
                             f["mu_sgs"])
    _compare(out, r, TOL32, "diffu reference-driver case")


def test_determinism_and_split_alias(cuda):
    host, dev = _case(cuda, 4, 4, jitter=0.05, mu=1e-3)
    a = [x.clone() for x in dev.convec()]
    b = [x.clone() for x in dev.convec(split=True)]
    for x, y in zip(a, b):
        assert refimpl.rel_l2(_cpu(x), _cpu(y)) < 1e-6
    c = [x.clone() for x in dev.diffu()]
    d = [x.clone() for x in dev.diffu()]
    for x, y in zip(c, d):
        assert refimpl.rel_l2(_cpu(x), _cpu(y)) < 1e-6


def test_outputs_are_intent_out(cuda):
    """Residual arrays are overwritten, not accumulated into."""
    host, dev = _case(cuda, 3, 2)
    ref = [x.clone() for x in dev.convec()]
    for x in (dev.Rmass, dev.Rmom, dev.Rener):
        x.fill_(123.0)
    out = dev.convec()
    for x, y in zip(out, ref):
        assert refimpl.rel_l2(_cpu(x), _cpu(y)) < 1e-6


def test_checked_mode_validation(cuda):
    host, dev = _case(cuda, 4, 2)
    P = 4
    kernels.check_element_tables(P, dev.nelem, dev.npoin, dev.connec, dev.dlxigp_ip, dev.invAtoIJK, dev.AtoI,
                                 dev.AtoJ, dev.AtoK)
    kernels.set_checked(True)
    try:
        dev.convec()
        bad = dev.dlxigp_ip.clone()
        bad[7] += 1.0
        with pytest.raises(capi.MsodError) as ei:
            kernels.check_element_tables(P, dev.nelem, dev.npoin, dev.connec, bad, dev.invAtoIJK, dev.AtoI,
                                         dev.AtoJ, dev.AtoK)
        assert ei.value.code == capi.MSOD_ERR_BAD_TABLES
        inv = dev.invAtoIJK.clone()
        inv[[0, 1]] = inv[[1, 0]]
        with pytest.raises(capi.MsodError) as ei:
            kernels.check_element_tables(P, dev.nelem, dev.npoin, dev.connec, dev.dlxigp_ip, inv, dev.AtoI,
                                         dev.AtoJ, dev.AtoK)
        assert ei.value.code == capi.MSOD_ERR_BAD_TABLES
        con = dev.connec.clone()
        con[5] = dev.npoin + 1
        with pytest.raises(capi.MsodError) as ei:
            kernels.full_convec_ijk(dev.nelem, dev.npoin, con, None, None, dev.He, dev.gpvol, dev.dlxigp_ip, None,
                                    dev.invAtoIJK, dev.AtoI, dev.AtoJ, dev.AtoK, dev.u, dev.q, dev.rho, dev.pr,
                                    dev.E, dev.Rmass, dev.Rmom, dev.Rener)
        assert ei.value.code == capi.MSOD_ERR_BAD_TABLES
    finally:
        kernels.set_checked(False)


def test_wrong_device_or_dtype_rejected(cuda):
    import torch

    host, dev = _case(cuda, 2, 2)
    with pytest.raises(ValueError):
        kernels.full_convec_ijk(*dev.geometry(), dev.u.cpu(), dev.q, dev.rho, dev.pr, dev.E, dev.Rmass, dev.Rmom,
                                dev.Rener)
    with pytest.raises(TypeError):
        kernels.full_convec_ijk(*dev.geometry(), dev.u.double(), dev.q, dev.rho, dev.pr, dev.E, dev.Rmass, dev.Rmom,
                                dev.Rener)
    del torch


def test_sampled_parity_plain_64(cuda):
    """The throughput workload (64^3 hexes, porder 4, jittered): a slab of 2048
    elements from the middle of the mesh against the oracle, and the whole mesh
    against the FP64 build (size-independent precision check)."""
    import torch

    host = workload.HostCase(workload.CONFIGS["plain_64"])
    dev = workload.DeviceCase(host, device=cuda)
    n = host.cfg.nnode
    e0, e1 = host.nelem // 2, host.nelem // 2 + 2048
    con = np.ascontiguousarray(host.connec.reshape(n, host.nelem)[:, e0:e1]).reshape(-1)
    He = _cpu(dev.He).reshape(host.nelem, -1)[e0:e1].reshape(-1)
    gp = _cpu(dev.gpvol).reshape(host.nelem, -1)[e0:e1].reshape(-1)
    geom = dict(host.tables, connec=con, He=He, gpvol=gp)
    d_con, d_He, d_gp = (torch.from_numpy(x).to(cuda) for x in (con, He, gp))
    ne = e1 - e0
    geo = (ne, dev.npoin, d_con, None, None, d_He, d_gp, dev.dlxigp_ip, None, dev.invAtoIJK, dev.AtoI, dev.AtoJ,
           dev.AtoK)
    kernels.full_convec_ijk(*geo, dev.u, dev.q, dev.rho, dev.pr, dev.E, dev.Rmass, dev.Rmom, dev.Rener)
    f = host.fields
    r = O.full_convec_ijk(4, ne, dev.npoin, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], nthreads=NTH)
    _compare((dev.Rmass, dev.Rmom, dev.Rener), r, TOL32, "convec plain_64 slab")
    mu = np.zeros(ne * n, np.float32)
    d_mu = torch.from_numpy(mu).to(cuda)
    kernels.full_diffusion_ijk(*geo, 1004.5, 0.71, dev.rho, dev.u, dev.Tem, dev.mu_fluid, d_mu, d_mu, dev.Dmass,
                               dev.Dmom, dev.Dener)
    r = O.full_diffusion_ijk(4, ne, dev.npoin, geom, 1004.5, 0.71, f["rho"], f["u"], f["Tem"], f["mu_fluid"], mu, mu,
                             nthreads=NTH)
    _compare((dev.Dmass, dev.Dmom, dev.Dener), r, TOL32, "diffu plain_64 slab")
    # whole mesh: FP32 kernels against the FP64 kernels on the same (FP32-rounded) inputs
    c32 = [x.clone() for x in dev.convec()]
    d32 = [x.clone() for x in dev.diffu()]
    f64 = {k: getattr(dev, k).double() for k in ("u", "q", "rho", "pr", "E", "Tem", "mu_fluid", "mu_e", "mu_sgs")}
    He64, gp64 = dev.He.double(), dev.gpvol.double()
    dl64 = torch.from_numpy(fem.element_tables(4, np.float64)["dlxigp_ip"]).to(cuda)
    geo64 = (dev.nelem, dev.npoin, dev.connec, None, None, He64, gp64, dl64, None, dev.invAtoIJK, dev.AtoI, dev.AtoJ,
             dev.AtoK)
    out = [torch.empty_like(x, dtype=torch.float64) for x in c32]
    kernels.full_convec_ijk(*geo64, f64["u"], f64["q"], f64["rho"], f64["pr"], f64["E"], *out)
    _compare(c32, [_cpu(x) for x in out], TOL32, "convec plain_64 fp32 vs fp64")
    kernels.full_diffusion_ijk(*geo64, 1004.5, 0.71, f64["rho"], f64["u"], f64["Tem"], f64["mu_fluid"], f64["mu_e"],
                               f64["mu_sgs"], *out)
    _compare(d32, [_cpu(x) for x in out], TOL32, "diffu plain_64 fp32 vs fp64")
