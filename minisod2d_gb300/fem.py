"""Host-side element setup, mesh and field recipes (numpy front end of libmsod).

Mirrors the setup half of the reference driver (main.f90:110-361): element
index maps and GLL basis tables, the mesh, the metric (on the device) and the
seeded node fields.
"""
import ctypes as C

import numpy as np

from . import capi


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def element_tables(porder, dtype=np.float32):
    """Tables of main.f90:110-255 as a dict of flat numpy arrays.

    invAtoIJK[(k*Q+j)*Q+i], AtoIJK, AtoI/J/K (1-based), xgp(ngaus,3),
    wgp(ngaus), Ngp(ngaus,nnode), dNgp(3,nnode,ngaus), dlxigp_ip(ngaus,3,Q).
    """
    P = int(porder)
    if P < 1 or P > capi.MSOD_MAX_PORDER:
        raise capi.MsodError(capi.MSOD_ERR_PORDER, "porder %d" % P)
    Q = P + 1
    n = Q ** 3
    t = dict(P=P, n=n)
    for k in ("invAtoIJK", "AtoIJK", "AtoI", "AtoJ", "AtoK"):
        t[k] = np.zeros(n, np.int32)
    t["xgp"] = np.zeros(3 * n, dtype)
    t["wgp"] = np.zeros(n, dtype)
    t["Ngp"] = np.zeros(n * n, dtype)
    t["dNgp"] = np.zeros(3 * n * n, dtype)
    t["dlxigp_ip"] = np.zeros(3 * n * Q, dtype)
    name = "msod_fem_element_tables" if np.dtype(dtype) == np.float32 else "msod_fem_element_tables_f64"
    capi.call(name, P, *[_p(t[k]) for k in ("invAtoIJK", "AtoIJK", "AtoI", "AtoJ", "AtoK", "xgp", "wgp", "Ngp",
                                            "dNgp", "dlxigp_ip")])
    return t


def structured_mesh(porder, nx, ny, nz, tables, jitter=0.0, seed=0, coords=True):
    """Structured shared-node hex mesh of the unit cube.

    Returns (connec[a*nelem+e] int32 1-based, coord[d*npoin+p] float32 or None,
    nelem, npoin).
    """
    P = int(porder)
    n = (P + 1) ** 3
    nelem = nx * ny * nz
    npoin = (nx * P + 1) * (ny * P + 1) * (nz * P + 1)
    connec = np.zeros(nelem * n, np.int32)
    coord = np.zeros(3 * npoin, np.float32) if coords else None
    capi.call("msod_mesh_structured", P, nx, ny, nz, _p(tables["AtoI"]), _p(tables["AtoJ"]), _p(tables["AtoK"]),
              float(jitter), int(seed) & (2 ** 64 - 1), _p(connec), _p(coord) if coords else None)
    return connec, coord, nelem, npoin


def fields_recipe(kind, nmodes, seed, npoin, coord):
    """Seeded FP32 node fields: dict rho, u(3*npoin), q, pr, E, Tem, mu_fluid."""
    f = {k: np.zeros(npoin, np.float32) for k in ("rho", "pr", "E", "Tem", "mu_fluid")}
    f["u"] = np.zeros(3 * npoin, np.float32)
    f["q"] = np.zeros(3 * npoin, np.float32)
    coord = np.ascontiguousarray(coord, np.float32)
    capi.call("msod_fields_recipe", int(kind), int(nmodes), int(seed) & (2 ** 64 - 1), int(npoin), _p(coord),
              _p(f["rho"]), _p(f["u"]), _p(f["q"]), _p(f["pr"]), _p(f["E"]), _p(f["Tem"]), _p(f["mu_fluid"]))
    return f


# ---------------------------------------------------------------------------
# Linear tetrahedra (the reference driver's TET04 data, main.f90:365-407)
# ---------------------------------------------------------------------------

def tet_element_tables(dtype=np.float32):
    """tet_4points + tet_04 tables: Ngp[a*4+g] (Ngp(igaus,inode)), dNgp[(g*4+a)*3+d],
    xgp[d*4+g], wgp[4]."""
    t = dict(Ngp=np.zeros(16, dtype), dNgp=np.zeros(48, dtype), xgp=np.zeros(12, dtype), wgp=np.zeros(4, dtype))
    name = "msod_tet_element_tables" if np.dtype(dtype) == np.float32 else "msod_tet_element_tables_f64"
    capi.call(name, _p(t["Ngp"]), _p(t["dNgp"]), _p(t["xgp"]), _p(t["wgp"]))
    return t


# xyzTET of the driver (main.f90:390-393) as xyzBase[d*4+a].
TET_BASE = np.array([0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1], np.float32)


def tet_mesh_disconnected(nelem, xyzBase=TET_BASE, coords=True):
    """The driver's disconnected tet mesh (gen_tet_mesh): (connec[a*nelem+e], coord or None, npoin = 4 nelem)."""
    connec = np.zeros(4 * nelem, np.int32)
    coord = np.zeros(3 * 4 * nelem, np.float32) if coords else None
    base = np.ascontiguousarray(xyzBase, np.float32)
    capi.call("msod_tet_mesh_disconnected", int(nelem), _p(base), _p(connec), _p(coord) if coords else None)
    return connec, coord, 4 * nelem


def mesh_disconnected(porder, nelem, tables, coords=True):
    """The reference driver's disconnected mesh (create_mesh with xyzBase = xgp):
    (connec[a*nelem+e], coord[d*npoin+p] or None, npoin = nelem*nnode)."""
    n = (int(porder) + 1) ** 3
    connec = np.zeros(nelem * n, np.int32)
    coord = np.zeros(3 * nelem * n, np.float32) if coords else None
    xgp = np.ascontiguousarray(tables["xgp"], np.float32)
    capi.call("msod_mesh_disconnected", int(porder), int(nelem), _p(xgp), _p(connec),
              _p(coord) if coords else None)
    return connec, coord, nelem * n


def reference_ic(porder, nelem, npoin, connec):
    """The reference driver's initial condition (main.f90:320-361) as FP32 arrays."""
    n = (int(porder) + 1) ** 3
    f = {k: np.zeros(npoin, np.float32) for k in ("rho", "pr", "E", "Tem", "mu_fluid")}
    f["u"] = np.zeros(3 * npoin, np.float32)
    f["q"] = np.zeros(3 * npoin, np.float32)
    f["mu_e"] = np.ones(nelem * n, np.float32)
    f["mu_sgs"] = np.ones(nelem * n, np.float32)
    c = np.ascontiguousarray(connec, np.int32)
    capi.call("msod_reference_ic", int(porder), int(nelem), int(npoin), _p(c), _p(f["u"]), _p(f["q"]), _p(f["rho"]),
              _p(f["pr"]), _p(f["E"]), _p(f["Tem"]), _p(f["mu_fluid"]), _p(f["mu_e"]), _p(f["mu_sgs"]))
    return f
