"""CPU checks of the linear-tetrahedron oracle and host setup.

The C oracle's restatement of fem_convec / fem_diffu / tet_jacobian
(elem_convec.f90:839-948, elem_diffu.f90:199-317, jacobian_oper.f90:138-267)
is pinned by known answers (the driver's unit tets, constant and linear
fields) and by the independently structured numpy restatement in
tests/refimpl.py.  The library's host tables and mesh must equal the
oracle's bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import refimpl as R


def _fields(npoin, nelem, seed=0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    f = dict(rho=1 + rng.random(npoin), pr=1 + rng.random(npoin), E=2 + rng.random(npoin),
             u=rng.standard_normal(3 * npoin), Tem=1 + rng.random(npoin), mu_fluid=0.1 * rng.random(npoin),
             mu_e=0.1 * rng.random(4 * nelem), mu_sgs=0.1 * rng.random(4 * nelem))
    f["q"] = (f["u"].reshape(3, -1) * f["rho"]).reshape(-1)
    return {k: v.astype(dtype) for k, v in f.items()}


def _mesh(kind, dtype=np.float64):
    t = O.tet_element_tables(dtype)
    if kind == "driver":
        nelem = 40
        connec, coord = O.gen_tet_mesh(nelem, dtype=dtype)
        npoin = 4 * nelem
    else:
        connec, coord, nelem, npoin = R.tet_mesh_shared(3, 0.2, 5)
        coord = coord.astype(dtype)
    He, gp = O.tet_jacobian(nelem, npoin, connec, coord, t["dNgp"], t["wgp"], dtype)
    return t, connec, coord, nelem, npoin, He, gp


def test_tet_tables_known_answers():
    t = O.tet_element_tables(np.float64)
    N = t["Ngp"].reshape(4, 4)  # N[a, g] = N_a(x_g)
    assert np.allclose(N.sum(0), 1.0, atol=1e-15)
    assert np.allclose(t["dNgp"].reshape(4, 4, 3).sum(1), 0.0)
    assert t["wgp"].sum() == 1.0
    x = t["xgp"].reshape(3, 4)  # x[d, g]
    # barycentric coordinates (1 - x - y - z, x, y, z) of every point: a permutation of (a, b, b, b)
    bary = np.vstack([1 - x.sum(0), x])
    assert np.allclose(np.sort(bary, 0), np.sort(bary, 0)[:, :1], atol=1e-15)
    assert np.allclose(np.sort(bary, 0)[:, 0], [0.1381966011250110] * 3 + [0.5854101966249680], atol=1e-15)
    assert np.argmax(x[:, 0]) == 0 and np.argmax(x[:, 1]) == 1 and np.argmax(x[:, 2]) == 2
    assert np.allclose(x[:, 3], 0.1381966011250110)


def test_library_tet_tables_and_mesh_equal_the_oracle():
    from minisod2d_gb300 import fem

    for dt in (np.float32, np.float64):
        a, b = fem.tet_element_tables(dt), O.tet_element_tables(dt)
        for k in ("Ngp", "dNgp", "xgp", "wgp"):
            assert np.array_equal(a[k], b[k]), k
    c, x, npoin = fem.tet_mesh_disconnected(9)
    oc, ox = O.gen_tet_mesh(9)
    assert npoin == 36 and np.array_equal(c, oc) and np.array_equal(x, ox)
    c2, x2, _ = fem.tet_mesh_disconnected(9, coords=False)
    assert np.array_equal(c2, oc) and x2 is None


def test_tet_jacobian_known_answers():
    t, connec, coord, nelem, npoin, He, gp = _mesh("driver")
    assert np.array_equal(He.reshape(nelem, 4, 3, 3), np.broadcast_to(np.eye(3), (nelem, 4, 3, 3)))
    assert np.all(gp == 0.25)
    t, connec, coord, nelem, npoin, He, gp = _mesh("shared")
    assert abs(gp.sum() - 6.0) < 1e-12 and np.all(gp > 0)  # weights sum to 1: gpvol = det = 6 volume
    # He is the inverse of Je = dN . x at every point
    con = connec.reshape(4, nelem).T - 1
    X = coord.reshape(3, npoin).T[con]                            # [e, a, d]
    dN = t["dNgp"].reshape(4, 4, 3)[0]                             # constant over the points
    Je = np.einsum("ai,ead->eid", dN, X)
    H = He.reshape(nelem, 4, 3, 3)[:, 0].transpose(0, 2, 1)       # H[e, i, j] = He(i, j)
    assert np.allclose(np.einsum("eij,ejk->eik", H, Je), np.eye(3), atol=1e-12)


@pytest.mark.parametrize("kind", ["driver", "shared"])
def test_tet_oracle_matches_numpy_restatement(kind):
    t, connec, coord, nelem, npoin, He, gp = _mesh(kind)
    f = _fields(npoin, nelem, seed=7)
    a = O.fem_convec(nelem, npoin, connec, t["Ngp"], t["dNgp"], He, gp, f["u"], f["q"], f["rho"], f["pr"], f["E"],
                     np.float64, nthreads=4)
    b = R.fem_convec(nelem, npoin, connec, t["Ngp"], t["dNgp"], He, gp, f["u"], f["q"], f["rho"], f["pr"], f["E"])
    for x, y in zip(a, b):
        assert R.rel_l2(x, y) < 1e-13
    a = O.fem_diffu(nelem, npoin, connec, t["Ngp"], t["dNgp"], He, gp, 1.0, 0.71, f["rho"], f["u"], f["Tem"],
                    f["mu_fluid"], f["mu_e"], f["mu_sgs"], np.float64, nthreads=4)
    b = R.fem_diffu(nelem, npoin, connec, t["Ngp"], t["dNgp"], He, gp, 1.0, 0.71, f["rho"], f["u"], f["Tem"],
                    f["mu_fluid"], f["mu_e"], f["mu_sgs"])
    for x, y in zip(a, b):
        assert R.rel_l2(x, y) < 1e-13


def test_tet_oracle_constant_fields_give_zero():
    t, connec, coord, nelem, npoin, He, gp = _mesh("shared")
    one = np.ones(npoin)
    u = np.concatenate([0.3 * one, -0.2 * one, 0.1 * one])
    for r in O.fem_convec(nelem, npoin, connec, t["Ngp"], t["dNgp"], He, gp, u, 1.2 * u, 1.2 * one, 0.8 * one,
                          2.5 * one, np.float64):
        assert np.abs(r).max() < 1e-13
    for r in O.fem_diffu(nelem, npoin, connec, t["Ngp"], t["dNgp"], He, gp, 1.0, 0.71, 1.2 * one, u, one, one,
                         np.ones(4 * nelem), np.ones(4 * nelem), np.float64):
        assert np.abs(r).max() < 1e-13


def test_tet_oracle_linear_density_mass_residual():
    """rho = x, u constant (q = rho u): every point has div q = u.grad rho = u_x, div u = 0,
    so Rmass(a) = sum_g gpvol(g) Ngp(g,a) 1/2 (u_x + u_x) accumulated over the elements of a."""
    t, connec, coord, nelem, npoin, He, gp = _mesh("shared")
    x = coord[:npoin]
    ux = 0.7
    u = np.concatenate([np.full(npoin, ux), np.zeros(npoin), np.zeros(npoin)])
    rho = 1.0 + x
    q = (u.reshape(3, -1) * rho).reshape(-1)
    Rm, _, _ = O.fem_convec(nelem, npoin, connec, t["Ngp"], t["dNgp"], He, gp, u, q, rho, np.ones(npoin),
                            np.ones(npoin), np.float64)
    expect = np.zeros(npoin)
    N = t["Ngp"].reshape(4, 4)  # N[a, g]
    con = connec.reshape(4, nelem).T - 1
    w = gp.reshape(nelem, 4) @ N.T  # [e, a] = sum_g gpvol(g) N_a(x_g)
    np.add.at(expect, con, w * ux)
    assert np.allclose(Rm, expect, rtol=1e-12, atol=1e-14)


def test_tet_oracle_fp32_floor():
    t32 = O.tet_element_tables(np.float32)
    t, connec, coord, nelem, npoin, He, gp = _mesh("shared", np.float32)
    f = _fields(npoin, nelem, seed=2, dtype=np.float32)
    a = O.fem_convec(nelem, npoin, connec, t32["Ngp"], t32["dNgp"], He, gp, f["u"], f["q"], f["rho"], f["pr"],
                     f["E"], np.float32)
    b = O.fem_convec(nelem, npoin, connec, t32["Ngp"], t32["dNgp"], He, gp, f["u"], f["q"], f["rho"], f["pr"],
                     f["E"], np.float64)
    for x, y in zip(a, b):
        assert R.rel_l2(x.astype(np.float64), y) < 1e-5
