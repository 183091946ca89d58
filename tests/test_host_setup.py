"""Host-side product code (no GPU): element tables, mesh, fields, C-ABI surface."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from minisod2d_gb300 import capi, fem
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bits(a):
    return a if a.dtype == np.int32 else a.view(np.uint8)


@pytest.mark.parametrize("P", range(1, 9))
def test_element_tables_bit_exact(msod_lib, P):
    """The library's tables equal the oracle's restatement of main.f90:110-255 bit for bit."""
    for dt in (np.float32, np.float64):
        t = fem.element_tables(P, dt)
        o = O.element_tables(P, dt)
        for k in ("invAtoIJK", "AtoIJK", "AtoI", "AtoJ", "AtoK", "xgp", "wgp", "Ngp", "dNgp", "dlxigp_ip"):
            assert np.array_equal(_bits(t[k]), _bits(o[k])), k


def test_header_symbols_exported(msod_lib):
    """Every function declared in include/msod.h is exported by libmsod.so and bound in capi."""
    hdr = open(os.path.join(ROOT, "include", "msod.h")).read()
    names = set(re.findall(r"\b(msod_[a-z0-9_]+)\s*\(", hdr))
    assert len(names) >= 20
    for name in names:
        assert hasattr(msod_lib, name), name
        assert name in capi.SIGNATURES, name


def test_invalid_arguments_rejected_on_host(msod_lib):
    """Argument errors are reported as codes before any device work."""
    L = capi.lib()
    args = [0] * 22 + [None]
    rc = L.msod_convec_ijk(9, 1, 1, *[None] * 19, None)
    assert rc == capi.MSOD_ERR_PORDER
    assert b"porder" in L.msod_last_error_string()
    rc = L.msod_convec_ijk(4, 0, 1, *[None] * 19, None)
    assert rc == capi.MSOD_ERR_INVALID_ARG
    dummy = C.c_void_p(16)
    geo = [dummy] * 11
    rc = L.msod_convec_ijk(4, 10, 100, dummy, None, None, dummy, dummy, dummy, None, dummy, dummy, dummy, dummy,
                           *[None] * 8, None)
    assert rc == capi.MSOD_ERR_INVALID_ARG
    rc = L.msod_diffusion_ijk(4, 1 << 30, 100, *[dummy] * 11, 1.0, 1.0, *[dummy] * 9, None)
    assert rc == capi.MSOD_ERR_INVALID_ARG  # nelem*nnode beyond int32
    rc = L.msod_diffusion_ijk(4, 10, 100, *[dummy] * 11, 1.0, 0.0, *[dummy] * 9, None)
    assert rc == capi.MSOD_ERR_INVALID_ARG  # Pr = 0
    del args, geo


def test_mesh_structure(msod_lib):
    P, nx = 4, 3
    t = fem.element_tables(P)
    connec, coord, ne, npn = fem.structured_mesh(P, nx, nx, nx, t, 0.0, 0)
    n = t["n"]
    assert ne == nx ** 3 and npn == (nx * P + 1) ** 3
    c = connec.reshape(n, ne)
    assert c.min() == 1 and c.max() == npn
    assert len(np.unique(c)) == npn  # every node used
    # each element's nodes are distinct
    assert all(len(np.unique(c[:, e])) == n for e in range(ne))
    # affine mesh: element nodes sit on the GLL points of the element box
    xg = t["xgp"].reshape(3, n)
    h = 1.0 / nx
    for e in (0, ne // 2, ne - 1):
        ex, ey, ez = e % nx, (e // nx) % nx, e // (nx * nx)
        p = c[:, e] - 1
        for d, o in enumerate((ex, ey, ez)):
            expect = (o + (xg[d] + 1) / 2) * h
            assert np.allclose(coord[d * npn + p], expect, atol=1e-6)
    # shared faces: neighbouring elements share exactly (P+1)^2 nodes
    assert len(np.intersect1d(c[:, 0], c[:, 1])) == (P + 1) ** 2


def test_mesh_jitter_bounds(msod_lib):
    P, nx = 2, 4
    t = fem.element_tables(P)
    _, c0, _, npn = fem.structured_mesh(P, nx, nx, nx, t, 0.0, 0)
    _, c1, _, _ = fem.structured_mesh(P, nx, nx, nx, t, 0.05, 0)
    _, c2, _, _ = fem.structured_mesh(P, nx, nx, nx, t, 0.05, 0)
    assert np.array_equal(c1, c2)  # seeded
    d = np.abs(c1 - c0).max()
    assert 0 < d <= 0.05 / nx + 1e-6
    assert c1.min() >= 0.0 and c1.max() <= 1.0


def test_mesh_errors(msod_lib):
    t = fem.element_tables(4)
    with pytest.raises(capi.MsodError):
        fem.structured_mesh(4, 0, 1, 1, t)
    with pytest.raises(capi.MsodError):
        fem.structured_mesh(4, 2, 2, 2, t, jitter=0.5)
    with pytest.raises(capi.MsodError):
        fem.element_tables(0)
    with pytest.raises(capi.MsodError):
        fem.element_tables(9)


def test_fields_recipe(msod_lib):
    P, nx = 4, 2
    t = fem.element_tables(P)
    _, coord, ne, npn = fem.structured_mesh(P, nx, nx, nx, t, 0.0, 0)
    f = fem.fields_recipe(0, 8, 0, npn, coord)
    x, y, z = (coord[d * npn:(d + 1) * npn].astype(np.float64) for d in range(3))
    rho = 1 + 0.1 * np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y) * np.sin(2 * np.pi * z)
    assert np.allclose(f["rho"], rho, atol=1e-6)
    assert np.allclose(f["pr"], 1 + 0.05 * np.cos(2 * np.pi * x), atol=1e-6)
    u = f["u"].reshape(3, npn)
    assert np.allclose(f["q"].reshape(3, npn), f["rho"] * u, rtol=1e-6)
    assert np.allclose(f["E"], f["pr"] / 0.4 / f["rho"] + 0.5 * (u ** 2).sum(0), rtol=1e-6)
    assert np.allclose(f["Tem"], f["pr"] / (f["rho"] * 287.0), rtol=1e-6)
    assert np.all(f["mu_fluid"] == np.float32(1.8e-5))
    f2 = fem.fields_recipe(0, 8, 0, npn, coord)
    assert all(np.array_equal(f[k], f2[k]) for k in f)
    f3 = fem.fields_recipe(0, 8, 1, npn, coord)
    assert not np.array_equal(f["u"], f3["u"])
    s = fem.fields_recipe(1, 8, 0, npn, coord)
    assert s["rho"].min() > 0.3 and s["rho"].max() < 1.7
    assert np.ptp(s["pr"]) == 0.0  # uniform pressure for the shock recipe


def test_no_device_is_reported(msod_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present")
    rc = capi.lib().msod_init(0)
    assert rc == capi.MSOD_ERR_NO_DEVICE


def test_mode_switch_arguments():
    """msod_set_mode: round trip through msod_get_mode, rejected values, back to the default."""
    from minisod2d_gb300 import capi, kernels

    try:
        assert kernels.get_mode() == ("fp32", "given")
        kernels.set_mode("fp16", "plain")
        assert kernels.get_mode() == ("fp16", "plain")
        with pytest.raises(capi.MsodError) as ei:
            capi.call("msod_set_mode", 7, 0, None)
        assert ei.value.code == capi.MSOD_ERR_INVALID_ARG
        with pytest.raises(capi.MsodError):
            capi.call("msod_set_mode", capi.MSOD_PREC_FP32, 9, None)
        with pytest.raises(capi.MsodError):  # the learned mode needs a network
            capi.call("msod_set_mode", capi.MSOD_PREC_FP32, capi.MSOD_MU_E_LEARNED, None)
        assert kernels.get_mode() == ("fp16", "plain")  # a rejected call changes nothing
    finally:
        kernels.set_mode()
    assert kernels.get_mode() == ("fp32", "given")


def test_one_call_and_time_update_arguments_rejected_on_host(msod_lib):
    """msod_convec_diffusion_ijk, msod_lumped_mass, msod_rk4_workspace_bytes and msod_rk4_step report
    argument errors as codes before any device work."""
    L = capi.lib()
    d = C.c_void_p(16)
    geo = [d, None, None, d, d, d, None, d, d, d, d]  # connec, Ngp, dNgp, He, gpvol, dlx, xgp, inv, AtoI/J/K
    fields = [d] * 9                                   # u, q, rho, pr, E, Tem, mu_fluid, mu_e, mu_sgs
    outs = [C.c_void_p(16 * (k + 1)) for k in range(6)]
    rc = L.msod_convec_diffusion_ijk(9, 10, 100, *geo, 1.0, 1.0, *fields, *outs, None)
    assert rc == capi.MSOD_ERR_PORDER
    rc = L.msod_convec_diffusion_ijk(4, 10, 100, *geo, 1.0, 0.0, *fields, *outs, None)
    assert rc == capi.MSOD_ERR_INVALID_ARG  # Pr = 0
    rc = L.msod_convec_diffusion_ijk(4, 10, 100, *geo, 1.0, 1.0, *fields[:5], None, *fields[6:], *outs, None)
    assert rc == capi.MSOD_ERR_INVALID_ARG  # NULL Tem
    alias = outs[:3] + [outs[0]] + outs[4:]
    rc = L.msod_convec_diffusion_ijk(4, 10, 100, *geo, 1.0, 1.0, *fields, *alias, None)
    assert rc == capi.MSOD_ERR_INVALID_ARG
    assert b"distinct" in L.msod_last_error_string()

    assert L.msod_lumped_mass(0, 10, 100, d, d, d, None) == capi.MSOD_ERR_PORDER
    assert L.msod_lumped_mass(4, 10, 100, d, None, d, None) == capi.MSOD_ERR_INVALID_ARG
    n = C.c_size_t(0)
    assert L.msod_rk4_workspace_bytes(0, C.byref(n)) == capi.MSOD_ERR_INVALID_ARG
    assert L.msod_rk4_workspace_bytes(100, C.byref(n)) == capi.MSOD_OK and n.value == 26 * 4 * 100
    g64 = [d, d, d, d, d, d, d, d]  # connec, He, gpvol, dlx, inv, AtoI/J/K
    phys = [1004.5, 0.71, 1.4, 287.0, d, d, d, d]  # Cp, Pr, gamma, Rgas, Ml, mu_fluid, mu_e, mu_sgs
    ws = C.c_void_p(4096)
    def step(P=4, nelem=10, dt=1e-3, w=ws, nbytes=n.value, gamma=1.4):
        ph = list(phys)
        ph[2] = gamma
        return L.msod_rk4_step(P, nelem, 100, *g64, *ph, dt, d, d, d, w, nbytes, None)
    assert step(P=9) == capi.MSOD_ERR_PORDER
    assert step(nelem=1 << 30) == capi.MSOD_ERR_INVALID_ARG       # nelem*nnode beyond int32
    assert step(dt=float("nan")) == capi.MSOD_ERR_INVALID_ARG
    assert step(gamma=1.0) == capi.MSOD_ERR_INVALID_ARG
    assert step(w=C.c_void_p(4097)) == capi.MSOD_ERR_INVALID_ARG  # not float-aligned
    assert step(nbytes=n.value - 4) == capi.MSOD_ERR_INVALID_ARG  # too small


def test_python_entry_points_have_no_cpu_path():
    """The Python mirror of the hot path refuses host tensors (the library has no CPU path) and
    wrong dtypes or sizes, before any library call."""
    import torch

    from minisod2d_gb300 import kernels

    P, nelem, npoin = 4, 2, 10
    n = (P + 1) ** 3
    f = lambda k, dt=torch.float32: torch.zeros(k, dtype=dt)
    i = lambda k: torch.ones(k, dtype=torch.int32)
    geo = (nelem, npoin, i(nelem * n), None, None, f(9 * nelem * n), f(nelem * n), f(3 * n * (P + 1)), None, i(n),
           i(n), i(n), i(n))
    fields = (f(3 * npoin), f(3 * npoin), f(npoin), f(npoin), f(npoin))
    outs = (f(npoin), f(3 * npoin), f(npoin))
    with pytest.raises(ValueError, match="CUDA tensor"):
        kernels.full_convec_ijk(*geo, *fields, *outs)
    with pytest.raises(ValueError, match="CUDA tensor"):
        kernels.full_diffusion_ijk(*geo, 1004.5, 0.71, f(npoin), f(3 * npoin), f(npoin), f(npoin), f(nelem * n),
                                   f(nelem * n), *outs)
    with pytest.raises(ValueError, match="CUDA tensor"):
        kernels.full_convec_diffusion_ijk(*geo, 1004.5, 0.71, *fields, f(npoin), f(npoin), f(nelem * n),
                                          f(nelem * n), *outs, f(npoin), f(3 * npoin), f(npoin))
    with pytest.raises(TypeError, match="float32"):
        kernels.full_convec_diffusion_ijk(*geo[:5], f(9 * nelem * n, torch.float64), *geo[6:], 1004.5, 0.71,
                                          *fields, f(npoin), f(npoin), f(nelem * n), f(nelem * n), *outs, f(npoin),
                                          f(3 * npoin), f(npoin))
    with pytest.raises(ValueError, match="not \\(porder\\+1\\)\\^3"):
        kernels.full_convec_ijk(*geo[:10], i(7), *geo[11:], *fields, *outs)
