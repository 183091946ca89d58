"""ctypes front end of the CPU oracle (test infrastructure only).

Wraps ``libmsod_oracle.so`` (built from ``msod_oracle.c`` by ``build.py``).
Arrays are numpy arrays in the reference's column-major layouts flattened to
1-D (see the header of ``msod_oracle.c``); ``dtype`` selects the FP32 (rp=4)
or FP64 (rp=8) build.  Only tests, ``__graft_entry__.smoke()`` and the CPU
legs of ``bench.py`` use this module.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        _build.build()
        _lib = C.CDLL(_build.LIB)
    return _lib


def _sfx(dtype):
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        return "_f32"
    if dtype == np.float64:
        return "_f64"
    raise ValueError("oracle dtype must be float32 or float64")


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _c(a, dtype):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a


def gll_weights_and_roots(P, dtype=np.float32):
    w = np.zeros(P + 1, dtype)
    r = np.zeros(P + 1, dtype)
    getattr(lib(), "orc_gll_weights_and_roots" + _sfx(dtype))(C.c_int(P), _p(w), _p(r))
    return w, r


def zelegl(P):
    et = np.zeros(P + 1)
    vn = np.zeros(P + 1)
    lib().orc_zelegl_f64(C.c_int(P), _p(et), _p(vn))
    return et, vn


def eval_lagrange_poly(P, xi, xp, dtype=np.float32, deriv=False):
    xi = _c(xi, dtype)
    out = np.zeros(P + 1, dtype)
    name = "orc_eval_lagrange_poly_deriv" if deriv else "orc_eval_lagrange_poly"
    f = getattr(lib(), name + _sfx(dtype))
    f.argtypes = [C.c_int, C.c_void_p, C.c_float if np.dtype(dtype) == np.float32 else C.c_double, C.c_void_p]
    f(P, _p(xi), xp, _p(out))
    return out


def gen_high_order_hex(P):
    t = np.zeros(((P + 1) ** 3, 3), np.int32)
    lib().orc_gen_high_order_hex_f32(C.c_int(P), _p(t))
    return t


def element_maps(P):
    """invAtoIJK (flat, [(k*Q+j)*Q+i]), AtoIJK, AtoI, AtoJ, AtoK -- 1-based."""
    Q = P + 1
    n = Q ** 3
    inv = np.zeros(n, np.int32)
    atoijk = np.zeros(n, np.int32)
    ai, aj, ak = (np.zeros(n, np.int32) for _ in range(3))
    rc = lib().orc_element_maps_f32(C.c_int(P), _p(inv), _p(atoijk), _p(ai), _p(aj), _p(ak))
    if rc != 0:
        raise RuntimeError("orc_element_maps failed")
    return inv, atoijk, ai, aj, ak


def element_tables(P, dtype=np.float32):
    """All per-element reference tables of main.f90:110-255."""
    inv, atoijk, ai, aj, ak = element_maps(P)
    n = (P + 1) ** 3
    xgp = np.zeros(3 * n, dtype)
    wgp = np.zeros(n, dtype)
    s = _sfx(dtype)
    getattr(lib(), "orc_gll_hex" + s)(C.c_int(P), _p(atoijk), _p(xgp), _p(wgp))
    Ngp = np.zeros(n * n, dtype)
    dNgp = np.zeros(3 * n * n, dtype)
    dlx = np.zeros(3 * n * (P + 1), dtype)
    getattr(lib(), "orc_element_basis" + s)(C.c_int(P), _p(atoijk), _p(xgp), _p(Ngp), _p(dNgp), _p(dlx))
    return dict(P=P, n=n, invAtoIJK=inv, AtoIJK=atoijk, AtoI=ai, AtoJ=aj, AtoK=ak,
                xgp=xgp, wgp=wgp, Ngp=Ngp, dNgp=dNgp, dlxigp_ip=dlx)


def elem_jacobian(P, nelem, npoin, connec, coord, dNgp, wgp, dtype=np.float32):
    n = (P + 1) ** 3
    gpvol = np.zeros(nelem * n, dtype)
    He = np.zeros(9 * nelem * n, dtype)
    getattr(lib(), "orc_elem_jacobian" + _sfx(dtype))(
        C.c_int(P), C.c_int(nelem), C.c_int(npoin), _p(_c(connec, np.int32)), _p(_c(coord, dtype)),
        _p(_c(dNgp, dtype)), _p(_c(wgp, dtype)), _p(gpvol), _p(He))
    return He, gpvol


def create_mesh_disconnected(P, nelem, xgp, dtype=np.float32):
    n = (P + 1) ** 3
    connec = np.zeros(nelem * n, np.int32)
    coord = np.zeros(3 * nelem * n, dtype)
    getattr(lib(), "orc_create_mesh_disconnected" + _sfx(dtype))(
        C.c_int(P), C.c_int(nelem), _p(_c(xgp, dtype)), _p(connec), _p(coord))
    return connec, coord


def structured_mesh(P, nx, tables, jitter=0.0, seed=0):
    """The benchmark workloads' structured shared-node mesh of the unit cube (nx^3 hexes):
    (connec[a*nelem+e] int32 1-based, coord[d*npoin+p] float32, nelem, npoin)."""
    n = (P + 1) ** 3
    nelem = nx ** 3
    npoin = (nx * P + 1) ** 3
    connec = np.zeros(nelem * n, np.int32)
    coord = np.zeros(3 * npoin, np.float32)
    f = lib().orc_mesh_structured_f32
    f.argtypes = [C.c_int] * 4 + [C.c_void_p] * 3 + [C.c_double, C.c_uint64, C.c_void_p, C.c_void_p]
    rc = f(P, nx, nx, nx, _p(_c(tables["AtoI"], np.int32)), _p(_c(tables["AtoJ"], np.int32)),
           _p(_c(tables["AtoK"], np.int32)), float(jitter), int(seed) & (2 ** 64 - 1), _p(connec), _p(coord))
    if rc:
        raise ValueError("orc_mesh_structured failed (%d)" % rc)
    return connec, coord, nelem, npoin


def fields_recipe(kind, nmodes, seed, npoin, coord):
    """The benchmark workloads' seeded node fields (FP32): dict of rho, u, q, pr, E, Tem, mu_fluid."""
    f = {k: np.zeros(npoin, np.float32) for k in ("rho", "pr", "E", "Tem", "mu_fluid")}
    f["u"] = np.zeros(3 * npoin, np.float32)
    f["q"] = np.zeros(3 * npoin, np.float32)
    fn = lib().orc_fields_recipe_f32
    fn.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_int64] + [C.c_void_p] * 8
    rc = fn(int(kind), int(nmodes), int(seed) & (2 ** 64 - 1), int(npoin), _p(_c(coord, np.float32)),
            _p(f["rho"]), _p(f["u"]), _p(f["q"]), _p(f["pr"]), _p(f["E"]), _p(f["Tem"]), _p(f["mu_fluid"]))
    if rc:
        raise ValueError("orc_fields_recipe failed (%d)" % rc)
    return f


def reference_ic(P, nelem, npoin, connec, dtype=np.float32):
    n = (P + 1) ** 3
    f = {k: np.zeros(npoin, dtype) for k in ("rho", "pr", "E", "Tem", "mu_fluid")}
    f["u"] = np.zeros(3 * npoin, dtype)
    f["q"] = np.zeros(3 * npoin, dtype)
    f["mu_e"] = np.zeros(nelem * n, dtype)
    f["mu_sgs"] = np.zeros(nelem * n, dtype)
    getattr(lib(), "orc_reference_ic" + _sfx(dtype))(
        C.c_int(P), C.c_int(nelem), C.c_int(npoin), _p(_c(connec, np.int32)), _p(f["u"]), _p(f["q"]),
        _p(f["rho"]), _p(f["pr"]), _p(f["E"]), _p(f["Tem"]), _p(f["mu_fluid"]), _p(f["mu_e"]), _p(f["mu_sgs"]))
    return f


def _geom_args(P, nelem, npoin, g, dtype):
    return [C.c_int(P), C.c_int(nelem), C.c_int(npoin), _p(g["connec"]), _p(g["He"]), _p(g["gpvol"]),
            _p(g["dlxigp_ip"]), _p(g["invAtoIJK"]), _p(g["AtoI"]), _p(g["AtoJ"]), _p(g["AtoK"])]


def _prep_geom(g, dtype):
    out = dict(g)
    for k in ("connec", "invAtoIJK", "AtoI", "AtoJ", "AtoK"):
        out[k] = _c(g[k], np.int32)
    for k in ("He", "gpvol", "dlxigp_ip"):
        out[k] = _c(g[k], dtype)
    return out


def full_convec_ijk(P, nelem, npoin, geom, u, q, rho, pr, E, dtype=np.float32, split=False, nthreads=1):
    """Rmass, Rmom (3*npoin, component-major), Rener."""
    g = _prep_geom(geom, dtype)
    ins = [_c(x, dtype) for x in (u, q, rho, pr, E)]
    Rmass = np.zeros(npoin, dtype)
    Rmom = np.zeros(3 * npoin, dtype)
    Rener = np.zeros(npoin, dtype)
    name = "orc_full_convec_ijk_split" if split else "orc_full_convec_ijk"
    rc = getattr(lib(), name + _sfx(dtype))(*_geom_args(P, nelem, npoin, g, dtype), *[_p(x) for x in ins],
                                          _p(Rmass), _p(Rmom), _p(Rener), C.c_int(nthreads))
    if rc != 0:
        raise RuntimeError(name + " failed")
    return Rmass, Rmom, Rener


def full_diffusion_ijk(P, nelem, npoin, geom, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs,
                       dtype=np.float32, nthreads=1):
    g = _prep_geom(geom, dtype)
    ins = [_c(x, dtype) for x in (rho, u, Tem, mu_fluid, mu_e, mu_sgs)]
    Rmass = np.zeros(npoin, dtype)
    Rmom = np.zeros(3 * npoin, dtype)
    Rener = np.zeros(npoin, dtype)
    real = C.c_float if np.dtype(dtype) == np.float32 else C.c_double
    rc = getattr(lib(), "orc_full_diffusion_ijk" + _sfx(dtype))(
        *_geom_args(P, nelem, npoin, g, dtype), real(Cp), real(Pr), *[_p(x) for x in ins],
        _p(Rmass), _p(Rmom), _p(Rener), C.c_int(nthreads))
    if rc != 0:
        raise RuntimeError("orc_full_diffusion_ijk failed")
    return Rmass, Rmom, Rener


def cpu_count():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def entropy_viscosity(P, nelem, npoin, geom, rho, u, pr, gamma=1.4, ce=0.1, cmax=0.5, normalise=True,
                      dtype=np.float64):
    """The library's entropy-viscosity estimator restated point by point: (mu_e, nu, numax)."""
    g = _prep_geom(geom, dtype)
    ins = [_c(x, dtype) for x in (rho, u, pr)]
    n = (P + 1) ** 3
    mu_e = np.zeros(nelem * n, dtype)
    nu = np.zeros(nelem, dtype)
    numax = np.zeros(nelem, dtype)
    real = C.c_float if np.dtype(dtype) == np.float32 else C.c_double
    rc = getattr(lib(), "orc_entropy_viscosity" + _sfx(dtype))(
        *_geom_args(P, nelem, npoin, g, dtype), *[_p(x) for x in ins], real(gamma), real(ce), real(cmax),
        C.c_int(1 if normalise else 0), _p(mu_e), _p(nu), _p(numax))
    if rc != 0:
        raise RuntimeError("orc_entropy_viscosity failed")
    return mu_e, nu, numax


# ---------------------------------------------------------------------------
# Time integration around the residuals.  The reference names a classical RK4
# with a lumped mass matrix (flag_rk_order = 4, flag_solver_type = 1,
# mod_numerical_params.f90:8,20) without containing either; restated in numpy
# on the oracle's residuals, as the library defines them (msod_rk.cu).
# ---------------------------------------------------------------------------
def lumped_mass(P, nelem, npoin, connec, gpvol, dtype=np.float64):
    """Ml(p) = sum of gpvol(e, g) over the element points g at node p."""
    n = (P + 1) ** 3
    ids = np.asarray(connec).reshape(n, nelem).T.reshape(-1) - 1  # element point (e, a) -> node
    Ml = np.zeros(npoin, dtype)
    np.add.at(Ml, ids, np.asarray(gpvol, dtype).reshape(-1))      # gpvol[e*n + a]
    return Ml


def rk4_step(P, nelem, npoin, geom, Cp, Pr, gamma, Rgas, Ml, mu_fluid, mu_e, mu_sgs, dt, rho, q, rhoE,
             dtype=np.float64, nthreads=1):
    """One classical RK4 step of dU/dt = -Ml^-1 (R_conv(U) + R_diff(U)), U = (rho, q = rho u, rhoE),
    the primitive fields derived per stage: u = q/rho, E = rhoE/rho, pr = (gamma-1)(rhoE - rho|u|^2/2),
    Tem = pr/(rho Rgas).  Returns the new (rho, q, rhoE)."""
    Ml = np.asarray(Ml, dtype)
    Ml3 = np.tile(Ml, 3)

    def rhs(r, qq, re):
        u = qq.reshape(3, npoin) / r
        E = re / r
        pr = (gamma - 1.0) * (re - 0.5 * r * (u * u).sum(0))
        Tem = pr / (r * Rgas)
        uf = np.ascontiguousarray(u.reshape(-1))
        cm, cq, ce = full_convec_ijk(P, nelem, npoin, geom, uf, qq, r, pr, E, dtype, nthreads=nthreads)
        dm, dq, de = full_diffusion_ijk(P, nelem, npoin, geom, Cp, Pr, r, uf, Tem, mu_fluid, mu_e, mu_sgs, dtype,
                                        nthreads=nthreads)
        return [-(cm + dm) / Ml, -(cq + dq) / Ml3, -(ce + de) / Ml]

    U0 = [np.asarray(x, dtype).copy() for x in (rho, q, rhoE)]
    k1 = rhs(*U0)
    k2 = rhs(*[a + 0.5 * dt * k for a, k in zip(U0, k1)])
    k3 = rhs(*[a + 0.5 * dt * k for a, k in zip(U0, k2)])
    k4 = rhs(*[a + dt * k for a, k in zip(U0, k3)])
    return [a + dt / 6.0 * (x1 + 2.0 * x2 + 2.0 * x3 + x4) for a, x1, x2, x3, x4 in zip(U0, k1, k2, k3, k4)]


# ---------------------------------------------------------------------------
# Linear tetrahedra (elem_tet.f90, quadrature_rules.f90:84-99, mod_mesh.f90:71-126,
# jacobian_oper.f90:138-267, elem_convec.f90:839-948, elem_diffu.f90:199-317)
# ---------------------------------------------------------------------------

def tet_element_tables(dtype=np.float32):
    """Ngp(4,4) (Ngp[a*4+g] = N_a(x_g)), dNgp(3,4,4), xgp(4,3), wgp(4): main.f90:377-383."""
    Ngp = np.zeros(16, dtype)
    dNgp = np.zeros(48, dtype)
    xgp = np.zeros(12, dtype)
    wgp = np.zeros(4, dtype)
    getattr(lib(), "orc_tet_element_tables" + _sfx(dtype))(_p(Ngp), _p(dNgp), _p(xgp), _p(wgp))
    return dict(Ngp=Ngp, dNgp=dNgp, xgp=xgp, wgp=wgp)


def gen_tet_mesh(nelem, xyzBase=None, dtype=np.float32):
    """The driver's disconnected tet mesh: npoin = 4 nelem (main.f90:386-394)."""
    if xyzBase is None:  # xyzTET, main.f90:390-393, as xyzBase[d*4+a]
        xyzBase = np.array([0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1], dtype)
    npoin = 4 * nelem
    connec = np.zeros(4 * nelem, np.int32)
    coord = np.zeros(3 * npoin, dtype)
    getattr(lib(), "orc_gen_tet_mesh" + _sfx(dtype))(C.c_int(nelem), C.c_int(npoin), _p(_c(xyzBase, dtype)),
                                                     _p(connec), _p(coord))
    return connec, coord


def tet_jacobian(nelem, npoin, connec, coord, dNgp, wgp, dtype=np.float32):
    gpvol = np.zeros(4 * nelem, dtype)
    He = np.zeros(36 * nelem, dtype)
    getattr(lib(), "orc_tet_jacobian" + _sfx(dtype))(
        C.c_int(nelem), C.c_int(npoin), _p(_c(connec, np.int32)), _p(_c(coord, dtype)), _p(_c(dNgp, dtype)),
        _p(_c(wgp, dtype)), _p(gpvol), _p(He))
    return He, gpvol


def fem_convec(nelem, npoin, connec, Ngp, dNgp, He, gpvol, u, q, rho, pr, E, dtype=np.float32, nthreads=1):
    ins = [_c(x, dtype) for x in (Ngp, dNgp, He, gpvol, u, q, rho, pr, E)]
    out = [np.zeros(n * npoin, dtype) for n in (1, 3, 1)]
    rc = getattr(lib(), "orc_fem_convec" + _sfx(dtype))(
        C.c_int(nelem), C.c_int(npoin), _p(_c(connec, np.int32)), *[_p(x) for x in ins], *[_p(x) for x in out],
        C.c_int(nthreads))
    if rc != 0:
        raise RuntimeError("orc_fem_convec failed")
    return tuple(out)


def fem_diffu(nelem, npoin, connec, Ngp, dNgp, He, gpvol, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs,
              dtype=np.float32, nthreads=1):
    a = [_c(x, dtype) for x in (Ngp, dNgp, He, gpvol)]
    b = [_c(x, dtype) for x in (rho, u, Tem, mu_fluid, mu_e, mu_sgs)]
    out = [np.zeros(n * npoin, dtype) for n in (1, 3, 1)]
    real = C.c_float if np.dtype(dtype) == np.float32 else C.c_double
    rc = getattr(lib(), "orc_fem_diffu" + _sfx(dtype))(
        C.c_int(nelem), C.c_int(npoin), _p(_c(connec, np.int32)), *[_p(x) for x in a], real(Cp), real(Pr),
        *[_p(x) for x in b], *[_p(x) for x in out], C.c_int(nthreads))
    if rc != 0:
        raise RuntimeError("orc_fem_diffu failed")
    return tuple(out)
