"""Known-answer tests that pin the CPU oracle (the reference has no tests of its own).

GLL nodes and weights against values computed from Legendre roots, the
derivative-matrix identities, the structure of the gmsh/SOD index maps, the
Jacobian of the reference's own test mesh (He = I, gpvol = wgp) and of affine
maps, zero residuals for constant fields, and exact residuals of polynomial
fields on affine meshes (where GLL collocation differentiates exactly).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import refimpl

GLL = {
    4: ([-1.0, -np.sqrt(3.0 / 7.0), 0.0, np.sqrt(3.0 / 7.0), 1.0], [1 / 10, 49 / 90, 32 / 45, 49 / 90, 1 / 10]),
    5: ([-1.0, -0.7650553239294647, -0.2852315164806451, 0.2852315164806451, 0.7650553239294647, 1.0],
        [1 / 15, 0.3784749562978470, 0.5548583770354863, 0.5548583770354863, 0.3784749562978470, 1 / 15]),
    7: ([-1.0, -0.8717401485096066, -0.5917001814331423, -0.2092992179024789, 0.2092992179024789,
         0.5917001814331423, 0.8717401485096066, 1.0],
        [1 / 28, 0.2107042271435061, 0.3411226924835044, 0.4124587946587038, 0.4124587946587038,
         0.3411226924835044, 0.2107042271435061, 1 / 28]),
}


@pytest.mark.parametrize("P", [4, 5, 7])
def test_gll_nodes_weights(P):
    w, x = O.gll_weights_and_roots(P, np.float64)
    xr, wr = GLL[P]
    assert np.allclose(x, xr, atol=1e-13)
    assert np.allclose(w, wr, atol=1e-13)
    w32, x32 = O.gll_weights_and_roots(P, np.float32)
    assert np.array_equal(x32, np.asarray(x, np.float32))
    assert abs(w.sum() - 2.0) < 1e-13


@pytest.mark.parametrize("P", range(1, 9))
def test_gll_general(P):
    w, x = O.gll_weights_and_roots(P, np.float64)
    assert abs(w.sum() - 2.0) < 1e-12
    assert np.all(np.diff(x) > 0)
    # exact for polynomials of degree <= 2P-1
    for deg in range(2 * P):
        exact = 0.0 if deg % 2 else 2.0 / (deg + 1)
        assert abs((w * x ** deg).sum() - exact) < 1e-12


@pytest.mark.parametrize("P", range(1, 9))
def test_derivative_matrix_identities(P):
    t = O.element_tables(P, np.float64)
    inv, D = refimpl.lattice_maps(t)
    w, x = O.gll_weights_and_roots(P, np.float64)
    # SOD order of the 1-D nodes: [0, P, 1, ..., P-1]
    sod = np.array([0, P] + list(range(1, P)))
    xs = x[sod]
    for d in range(3):
        assert np.allclose(D[d].sum(1), 0.0, atol=1e-11)       # derivative of a constant
        assert np.allclose(D[d] @ xs, 1.0, atol=1e-11)         # derivative of x
        for deg in range(2, P + 1):
            assert np.allclose(D[d] @ xs ** deg, deg * xs ** (deg - 1), atol=1e-9)
    # The per-point table is the 1-D matrix replicated along the other indices.
    Q = P + 1
    n = Q ** 3
    dl = t["dlxigp_ip"].reshape(Q, 3, n)
    for g in range(n):
        I, J, K = t["AtoI"][g] - 1, t["AtoJ"][g] - 1, t["AtoK"][g] - 1
        assert np.array_equal(dl[:, 0, g], D[0, I])
        assert np.array_equal(dl[:, 1, g], D[1, J])
        assert np.array_equal(dl[:, 2, g], D[2, K])


@pytest.mark.parametrize("P", range(1, 9))
def test_index_maps(P):
    inv, atoijk, ai, aj, ak = O.element_maps(P)
    Q = P + 1
    n = Q ** 3
    assert sorted(inv) == list(range(1, n + 1))
    assert sorted(atoijk) == list(range(1, n + 1))
    lat = inv.reshape(Q, Q, Q)
    for a in range(n):
        assert lat[ak[a] - 1, aj[a] - 1, ai[a] - 1] == a + 1
    # gmsh corners (mod_gmsh_indices.f90:19-30) relabelled 0 -> 1, P -> 2
    corners = [(1, 1, 1), (2, 1, 1), (2, 2, 1), (1, 2, 1), (1, 1, 2), (2, 1, 2), (2, 2, 2), (1, 2, 2)]
    for a, c in enumerate(corners[: min(8, n)]):
        assert (ai[a], aj[a], ak[a]) == c
    # AtoIJK follows the loop order k, i, j of main.f90:168-185
    c = 0
    for k in range(Q):
        for i in range(Q):
            for j in range(Q):
                assert atoijk[c] == lat[k, j, i]
                c += 1


def test_reference_mesh_jacobian():
    """Q4: the reference mesh copies the GLL cube, so He = I and gpvol = wgp."""
    P = 4
    t = O.element_tables(P, np.float64)
    ne = 2
    connec, coord = O.create_mesh_disconnected(P, ne, t["xgp"], np.float64)
    He, gp = O.elem_jacobian(P, ne, ne * t["n"], connec, coord, t["dNgp"], t["wgp"], np.float64)
    assert np.allclose(He.reshape(-1, 3, 3), np.eye(3), atol=1e-12)
    assert np.allclose(gp.reshape(ne, -1), t["wgp"], atol=1e-14)


@pytest.mark.parametrize("P", [2, 4])
def test_affine_jacobian(P):
    """x = A xi + b: Je = A^T (Je(i,j) = dx_j/dxi_i), He = Je^-1, gpvol = w det A."""
    t = O.element_tables(P, np.float64)
    A = np.array([[2.0, 0.3, 0.1], [0.2, 1.5, -0.4], [0.0, 0.25, 0.8]])
    b = np.array([0.5, -1.0, 2.0])
    n = t["n"]
    xi = t["xgp"].reshape(3, n).T
    x = xi @ A.T + b
    connec = np.arange(1, n + 1, dtype=np.int32)
    coord = x.T.reshape(-1).copy()
    He, gp = O.elem_jacobian(P, 1, n, connec, coord, t["dNgp"], t["wgp"], np.float64)
    Je = A.T
    Hm = np.swapaxes(He.reshape(n, 3, 3), 1, 2)  # [g, i, j] = He(i,j)
    assert np.allclose(Hm, np.linalg.inv(Je), atol=1e-12)
    assert np.allclose(gp, t["wgp"] * np.linalg.det(A), atol=1e-12)


def _structured(P, nx, jitter=0.0, dtype=np.float64, seed=3):
    """Small structured mesh built by the oracle-side routines only."""
    from minisod2d_gb300 import fem

    t = O.element_tables(P, dtype)
    t32 = fem.element_tables(P)
    connec, coord, nelem, npoin = fem.structured_mesh(P, nx, nx, nx, t32, jitter, seed)
    coord = coord.astype(dtype)
    He, gp = O.elem_jacobian(P, nelem, npoin, connec, coord, t["dNgp"], t["wgp"], dtype)
    geom = dict(t, connec=connec, He=He, gpvol=gp)
    return t, geom, nelem, npoin, coord


def test_constant_fields_zero_residuals():
    P, nx = 3, 2
    t, geom, ne, npn, coord = _structured(P, nx, jitter=0.05)
    one = np.ones(npn)
    u = np.concatenate([0.3 * one, -0.2 * one, 0.1 * one])
    q = 1.2 * u
    Rm, Rmom, Re = O.full_convec_ijk(P, ne, npn, geom, u, q, 1.2 * one, 0.9 * one, 2.5 * one, np.float64)
    for r in (Rm, Rmom, Re):
        assert np.abs(r).max() < 1e-12
    n = t["n"]
    mu = np.full(ne * n, 0.3)
    Dm, Dmom, De = O.full_diffusion_ijk(P, ne, npn, geom, 1004.5, 0.71, 1.2 * one, u, 0.7 * one, 1.8e-5 * one, mu,
                                        mu, np.float64)
    for r in (Dm, Dmom, De):
        assert np.abs(r).max() < 1e-10


def _poly_fields(coord, npoin):
    x, y, z = coord[:npoin], coord[npoin:2 * npoin], coord[2 * npoin:]
    rho = 1.0 + 0.1 * x - 0.05 * y + 0.02 * z
    u = np.concatenate([0.2 + 0.1 * y - 0.05 * z, -0.1 + 0.07 * x + 0.03 * z, 0.05 - 0.04 * x + 0.06 * y])
    q = np.concatenate([0.3 - 0.02 * z, 0.1 + 0.05 * x, -0.2 + 0.01 * y])
    pr = 1.0 + 0.03 * x + 0.02 * y - 0.01 * z
    E = 2.5 - 0.1 * x + 0.05 * z
    return rho, u, q, pr, E


def test_polynomial_convection_exact():
    """Linear fields on an affine mesh: every differentiated product has degree <= 4
    per variable, so P=4 collocation is exact and R(p) = density(x_p) * sum_e gpvol."""
    sympy = pytest.importorskip("sympy")
    P, nx = 4, 2
    t, geom, ne, npn, coord = _structured(P, nx)
    rho, u, q, pr, E = _poly_fields(coord, npn)
    Rm, Rmom, Re = O.full_convec_ijk(P, ne, npn, geom, u, q, rho, pr, E, np.float64)
    X, Y, Z = sympy.symbols("x y z")
    r_ = 1 + sympy.Rational(1, 10) * X - sympy.Rational(1, 20) * Y + sympy.Rational(1, 50) * Z
    U_ = [sympy.Rational(1, 5) + sympy.Rational(1, 10) * Y - sympy.Rational(1, 20) * Z,
          -sympy.Rational(1, 10) + sympy.Rational(7, 100) * X + sympy.Rational(3, 100) * Z,
          sympy.Rational(1, 20) - sympy.Rational(1, 25) * X + sympy.Rational(3, 50) * Y]
    Q_ = [sympy.Rational(3, 10) - sympy.Rational(1, 50) * Z, sympy.Rational(1, 10) + sympy.Rational(1, 20) * X,
          -sympy.Rational(1, 5) + sympy.Rational(1, 100) * Y]
    p_ = 1 + sympy.Rational(3, 100) * X + sympy.Rational(1, 50) * Y - sympy.Rational(1, 100) * Z
    E_ = sympy.Rational(5, 2) - sympy.Rational(1, 10) * X + sympy.Rational(1, 20) * Z
    xs = (X, Y, Z)
    k_ = sum(c * c for c in U_) / 2
    H_ = E_ + k_

    def div(V):
        return sum(sympy.diff(V[i], xs[i]) for i in range(3))

    divU, divQ = div(U_), div(Q_)
    dens_m = sympy.Rational(1, 2) * (divQ + r_ * divU) + sympy.Rational(1, 2) * sum(U_[i] * sympy.diff(r_, xs[i]) for i in range(3))
    dens_mom = []
    for i in range(3):
        divF = sum(sympy.diff(Q_[i] * U_[j], xs[j]) for j in range(3))
        divFuu = sum(sympy.diff(U_[i] * U_[j], xs[j]) for j in range(3))
        s = sympy.Rational(1, 4) * (divF + U_[i] * divQ + Q_[i] * divU + r_ * divFuu) + sympy.diff(p_, xs[i])
        s += sympy.Rational(1, 4) * sum(U_[i] * U_[j] * sympy.diff(r_, xs[j]) + Q_[j] * sympy.diff(U_[i], xs[j])
                                        + U_[j] * sympy.diff(Q_[i], xs[j]) for j in range(3))
        dens_mom.append(s)
    dens_e = sympy.Rational(1, 4) * (div([r_ * H_ * c for c in U_]) + H_ * divQ + r_ * H_ * divU + r_ * div([H_ * c for c in U_]))
    dens_e += sympy.Rational(1, 4) * sum(Q_[i] * sympy.diff(H_, xs[i]) + U_[i] * sympy.diff(r_ * H_, xs[i])
                                         + H_ * U_[i] * sympy.diff(r_, xs[i]) for i in range(3))
    f_m = sympy.lambdify(xs, dens_m, "numpy")
    f_mom = [sympy.lambdify(xs, s, "numpy") for s in dens_mom]
    f_e = sympy.lambdify(xs, dens_e, "numpy")
    M = refimpl.lumped_mass(geom, ne, npn, t["n"])
    xx, yy, zz = coord[:npn], coord[npn:2 * npn], coord[2 * npn:]
    assert np.allclose(Rm / M, f_m(xx, yy, zz), rtol=1e-9, atol=1e-11)
    for c in range(3):
        assert np.allclose(Rmom[c * npn:(c + 1) * npn] / M, f_mom[c](xx, yy, zz), rtol=1e-9, atol=1e-11)
    assert np.allclose(Re / M, f_e(xx, yy, zz), rtol=1e-9, atol=1e-11)


def test_linear_diffusion_interior():
    """Linear u, T, rho with constant viscosities on an affine mesh: the fluxes
    grad rho, grad T and tau are constant, tau.u is linear, so at interior nodes
    Dmass = Dmom = 0 and Dener = -(tau : grad u) * (lumped mass)."""
    P, nx = 4, 3
    t, geom, ne, npn, coord = _structured(P, nx)
    rho, u, q, pr, E = _poly_fields(coord, npn)
    T = 0.003 + 0.001 * coord[:npn]
    n = t["n"]
    mu_e = np.full(ne * n, 0.02)
    mu_sgs = np.zeros(ne * n)
    muf = np.full(npn, 1.8e-5)
    Cp, Pr = 1004.5, 0.71
    Dm, Dmom, De = O.full_diffusion_ijk(P, ne, npn, geom, Cp, Pr, rho, u, T, muf, mu_e, mu_sgs, np.float64)
    G = np.array([[0.0, 0.1, -0.05], [0.07, 0.0, 0.03], [-0.04, 0.06, 0.0]])  # d u_i / d x_j
    mu_f, mu_t = 1.8e-5, 1.8e-5 + 0.02
    tau = mu_t * (G + G.T) - mu_f * 2 / 3 * np.trace(G) * np.eye(3)
    c0 = (tau * G).sum()
    M = refimpl.lumped_mass(geom, ne, npn, n)
    NX = nx * P + 1
    idx = np.arange(npn)
    I, J, K = idx % NX, (idx // NX) % NX, idx // (NX * NX)
    interior = (I > 0) & (I < NX - 1) & (J > 0) & (J < NX - 1) & (K > 0) & (K < NX - 1)
    scale = np.abs(De).max()
    assert np.abs(Dm[interior]).max() < 1e-12
    for c in range(3):
        assert np.abs(Dmom[c * npn:(c + 1) * npn][interior]).max() < 1e-12
    assert np.allclose(De[interior], -c0 * M[interior], rtol=1e-9, atol=1e-12 * scale)


def test_fused_and_split_agree():
    """The fused and split reference kernels differ only in rounding."""
    P, nx = 4, 2
    from minisod2d_gb300 import fem

    t, geom, ne, npn, coord = _structured(P, nx, jitter=0.05, dtype=np.float32)
    f = fem.fields_recipe(0, 8, 1, npn, coord)
    a = O.full_convec_ijk(P, ne, npn, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], np.float32)
    b = O.full_convec_ijk(P, ne, npn, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], np.float32, split=True)
    for x, y in zip(a, b):
        assert refimpl.rel_l2(x, y) < 1e-5
    assert np.array_equal(a[0], b[0])  # the mass kernels are identical operation for operation
    assert np.array_equal(a[2], b[2])  # Rener is the split kernel's in both


def test_openmp_matches_serial():
    P, nx = 4, 2
    from minisod2d_gb300 import fem

    t, geom, ne, npn, coord = _structured(P, nx, jitter=0.05, dtype=np.float64)
    f = fem.fields_recipe(0, 8, 2, npn, coord.astype(np.float32))
    a = O.full_convec_ijk(P, ne, npn, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], np.float64, nthreads=1)
    b = O.full_convec_ijk(P, ne, npn, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], np.float64, nthreads=4)
    for x, y in zip(a, b):
        assert refimpl.rel_l2(x, y) < 1e-13


@pytest.mark.parametrize("P,nx,jitter,kind,nmodes,seed", [(4, 5, 0.05, 0, 8, 0), (5, 4, 0.05, 1, 8, 2024),
                                                           (7, 3, 0.05, 0, 16, 3), (2, 6, 0.0, 1, 8, 7)])
def test_oracle_workload_recipe_equals_library(P, nx, jitter, kind, nmodes, seed):
    """The oracle's restatement of the structured mesh and seeded fields (used by the benchmark's
    reference arm, which loads no product code) gives the library's setup bit for bit."""
    from minisod2d_gb300 import fem

    t = O.element_tables(P)
    c1, x1, ne1, np1 = O.structured_mesh(P, nx, t, jitter, seed)
    tl = fem.element_tables(P)
    c2, x2, ne2, np2 = fem.structured_mesh(P, nx, nx, nx, tl, jitter, seed)
    assert (ne1, np1) == (ne2, np2)
    assert np.array_equal(c1, c2)
    assert np.array_equal(x1.view(np.uint32), x2.view(np.uint32))
    f1 = O.fields_recipe(kind, nmodes, seed, np1, x1)
    f2 = fem.fields_recipe(kind, nmodes, seed, np2, x2)
    assert set(f1) == set(f2)
    for k in f1:
        assert np.array_equal(f1[k].view(np.uint32), f2[k].view(np.uint32)), k
