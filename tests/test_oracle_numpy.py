"""Cross-check of the C oracle against the independent numpy restatement (FP64)."""
import numpy as np
import pytest

from minisod2d_gb300 import fem
from oracle import oracle as O
from tests import refimpl


def _case(P, nx, jitter, kind=0, seed=5, mu=0.0):
    t = O.element_tables(P, np.float64)
    t32 = fem.element_tables(P)
    connec, coord, nelem, npoin = fem.structured_mesh(P, nx, nx, nx, t32, jitter, seed)
    He, gp = O.elem_jacobian(P, nelem, npoin, connec, coord.astype(np.float64), t["dNgp"], t["wgp"], np.float64)
    geom = dict(t, connec=connec, He=He, gpvol=gp)
    f = {k: v.astype(np.float64) for k, v in fem.fields_recipe(kind, 8, seed, npoin, coord).items()}
    rng = np.random.default_rng(seed)
    n = t["n"]
    f["mu_e"] = mu * rng.random(nelem * n)
    f["mu_sgs"] = mu * 0.5 * rng.random(nelem * n)
    return t, geom, nelem, npoin, f


@pytest.mark.parametrize("P,nx,jitter,kind", [(1, 3, 0.1, 0), (2, 2, 0.1, 1), (4, 2, 0.05, 0), (5, 1, 0.0, 1),
                                              (7, 1, 0.08, 0)])
def test_convection_c_vs_numpy(P, nx, jitter, kind):
    t, geom, ne, npn, f = _case(P, nx, jitter, kind)
    a = O.full_convec_ijk(P, ne, npn, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], np.float64)
    b = refimpl.convec(t, geom, ne, npn, f["u"], f["q"], f["rho"], f["pr"], f["E"])
    for x, y in zip(a, b):
        assert refimpl.rel_l2(x, y) < 1e-11


@pytest.mark.parametrize("P,nx,jitter,kind,mu", [(1, 3, 0.1, 0, 0.0), (2, 2, 0.1, 1, 1e-3), (4, 2, 0.05, 0, 1e-3),
                                                 (5, 1, 0.0, 1, 1e-2), (7, 1, 0.08, 0, 1e-3)])
def test_diffusion_c_vs_numpy(P, nx, jitter, kind, mu):
    t, geom, ne, npn, f = _case(P, nx, jitter, kind, mu=mu)
    a = O.full_diffusion_ijk(P, ne, npn, geom, 1004.5, 0.71, f["rho"], f["u"], f["Tem"], f["mu_fluid"], f["mu_e"],
                             f["mu_sgs"], np.float64)
    b = refimpl.diffusion(t, geom, ne, npn, 1004.5, 0.71, f["rho"], f["u"], f["Tem"], f["mu_fluid"], f["mu_e"],
                          f["mu_sgs"])
    for x, y in zip(a, b):
        if np.linalg.norm(y) == 0.0:
            assert np.abs(x).max() == 0.0
        else:
            assert refimpl.rel_l2(x, y) < 1e-11


def test_fp32_oracle_floor():
    """The FP32 oracle stays within 1e-5 of the FP64 oracle on a jittered smooth case:
    the noise floor under which FP32 implementations can be compared."""
    P, nx = 4, 2
    t64, geom64, ne, npn, f = _case(P, nx, 0.05, 0, mu=1e-3)
    t32 = O.element_tables(P, np.float32)
    geom32 = dict(t32, connec=geom64["connec"], He=geom64["He"].astype(np.float32),
                  gpvol=geom64["gpvol"].astype(np.float32))
    f32 = {k: v.astype(np.float32) for k, v in f.items()}
    a64 = O.full_convec_ijk(P, ne, npn, geom64, f32["u"], f32["q"], f32["rho"], f32["pr"], f32["E"], np.float64)
    a32 = O.full_convec_ijk(P, ne, npn, geom32, f32["u"], f32["q"], f32["rho"], f32["pr"], f32["E"], np.float32)
    for x, y in zip(a32, a64):
        assert refimpl.rel_l2(x, y) < 1e-5
    d64 = O.full_diffusion_ijk(P, ne, npn, geom64, 1004.5, 0.71, f32["rho"], f32["u"], f32["Tem"], f32["mu_fluid"],
                               f32["mu_e"], f32["mu_sgs"], np.float64)
    d32 = O.full_diffusion_ijk(P, ne, npn, geom32, 1004.5, 0.71, f32["rho"], f32["u"], f32["Tem"], f32["mu_fluid"],
                               f32["mu_e"], f32["mu_sgs"], np.float32)
    for x, y in zip(d32, d64):
        assert refimpl.rel_l2(x, y) < 1e-5
