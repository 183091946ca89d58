"""Independent numpy restatement of the hex convection/diffusion residuals.

A second CPU statement of the reference's mathematics (elem_convec.f90:198-431
with the energy terms of :674-832; elem_diffu.f90:10-197), written in a
different structure from the C oracle: whole-mesh lattice arrays, the 1-D
derivative matrices collapsed out of dlxigp_ip, einsum contractions, FP64
throughout.  Tests use it to cross-check the C oracle's transcription.
"""
import numpy as np


def lattice_maps(tables):
    P = tables["P"]
    Q = P + 1
    n = Q ** 3
    inv = tables["invAtoIJK"].reshape(Q, Q, Q) - 1  # [K, J, I] -> gmsh node
    dl = tables["dlxigp_ip"].astype(np.float64).reshape(Q, 3, n)  # [ii, d, g]
    D = np.zeros((3, Q, Q))
    for r in range(Q):
        D[0, r] = dl[:, 0, inv[0, 0, r]]
        D[1, r] = dl[:, 1, inv[0, r, 0]]
        D[2, r] = dl[:, 2, inv[r, 0, 0]]
    return inv, D


def _gather(geom, nelem, tables):
    P = tables["P"]
    Q = P + 1
    n = Q ** 3
    inv, D = lattice_maps(tables)
    nodes = (geom["connec"].reshape(n, nelem)[inv] - 1).transpose(3, 0, 1, 2)  # [e,K,J,I]
    H = geom["He"].astype(np.float64).reshape(nelem, n, 3, 3)[:, inv]  # [e,K,J,I,j,i]
    Hm = np.swapaxes(H, -1, -2)  # Hm[..., i, j] = He(i, j)
    gp = geom["gpvol"].astype(np.float64).reshape(nelem, n)[:, inv]
    return inv, D, nodes, Hm, gp


def _iso(D, f):
    """Iso-parametric derivatives of lattice field f[e,K,J,I] -> [..., 3]."""
    gx = np.einsum("rc,ekjc->ekjr", D[0], f)
    gy = np.einsum("rc,ekcI->ekrI", D[1], f)
    gz = np.einsum("rc,ecjI->erjI", D[2], f)
    return np.stack([gx, gy, gz], axis=-1)


def _grad(Hm, g):
    return np.einsum("...ij,...j->...i", Hm, g)


def convec(tables, geom, nelem, npoin, u, q, rho, pr, E):
    inv, D, nodes, Hm, gp = _gather(geom, nelem, tables)
    U = np.stack([u[c * npoin:(c + 1) * npoin] for c in range(3)], -1).astype(np.float64)[nodes]
    Qv = np.stack([q[c * npoin:(c + 1) * npoin] for c in range(3)], -1).astype(np.float64)[nodes]
    r = rho.astype(np.float64)[nodes]
    p = pr.astype(np.float64)[nodes]
    Ee = E.astype(np.float64)[nodes]
    k = 0.5 * (U ** 2).sum(-1)

    def grad_s(f):
        return _grad(Hm, _iso(D, f))

    def grad_v(V):  # gradV[..., i, j] = d V_i / d x_j
        return np.stack([grad_s(V[..., i]) for i in range(3)], axis=-2)

    def div_v(V):
        return np.trace(grad_v(V), axis1=-2, axis2=-1)

    gR, gP, gE, gRE, gk, gRk = (grad_s(f) for f in (r, p, Ee, r * Ee, k, r * k))
    gU, gQ = grad_v(U), grad_v(Qv)
    divU = np.trace(gU, axis1=-2, axis2=-1)
    divQ = np.trace(gQ, axis1=-2, axis2=-1)
    F = Qv[..., :, None] * U[..., None, :]
    Fuu = U[..., :, None] * U[..., None, :]
    divF = np.stack([div_v(F[..., i, :]) for i in range(3)], -1)
    divFuu = np.stack([div_v(Fuu[..., i, :]) for i in range(3)], -1)
    divFe = div_v((r * Ee)[..., None] * U)
    divFue = div_v(Ee[..., None] * U)
    divFk = div_v((r * k)[..., None] * U)
    divFuk = div_v(k[..., None] * U)
    Rm = 0.5 * (divQ + r * divU) + 0.5 * (U * gR).sum(-1)
    Rmom = (0.25 * (divF + U * divQ[..., None] + Qv * divU[..., None] + r[..., None] * divFuu) + gP
            + 0.25 * (U * (U * gR).sum(-1)[..., None] + np.einsum("...j,...ij->...i", Qv, gU)
                      + np.einsum("...j,...ij->...i", U, gQ)))
    Re = (0.25 * (divFe + Ee * divQ + r * Ee * divU + r * divFue) + 0.25 * (divFk + k * divQ + r * k * divU + r * divFuk)
          + 0.25 * ((Qv * gE).sum(-1) + (U * gRE).sum(-1) + Ee * (U * gR).sum(-1))
          + 0.25 * ((Qv * gk).sum(-1) + (U * gRk).sum(-1) + k * (U * gR).sum(-1)))
    out_m = np.zeros(npoin)
    out_mom = np.zeros((3, npoin))
    out_e = np.zeros(npoin)
    np.add.at(out_m, nodes, gp * Rm)
    for c in range(3):
        np.add.at(out_mom[c], nodes, gp * Rmom[..., c])
    np.add.at(out_e, nodes, gp * Re)
    return out_m, out_mom.reshape(-1), out_e


def diffusion(tables, geom, nelem, npoin, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs):
    inv, D, nodes, Hm, gp = _gather(geom, nelem, tables)
    n = inv.size
    U = np.stack([u[c * npoin:(c + 1) * npoin] for c in range(3)], -1).astype(np.float64)[nodes]
    r = rho.astype(np.float64)[nodes]
    T = Tem.astype(np.float64)[nodes]
    muf = mu_fluid.astype(np.float64)[nodes]
    me = mu_e.astype(np.float64).reshape(n, nelem)[inv].transpose(3, 0, 1, 2)
    ms = mu_sgs.astype(np.float64).reshape(n, nelem)[inv].transpose(3, 0, 1, 2)
    gR = _grad(Hm, _iso(D, r))
    gT = _grad(Hm, _iso(D, T))
    gU = np.stack([_grad(Hm, _iso(D, U[..., i])) for i in range(3)], axis=-2)
    divU = np.trace(gU, axis1=-2, axis2=-1)
    mu_f = muf + r * ms
    S = gU + np.swapaxes(gU, -1, -2)
    tau = (mu_f + me)[..., None, None] * S - (mu_f * 2.0 / 3.0 * divU)[..., None, None] * np.eye(3)
    tauU = np.einsum("...ij,...j->...i", tau, U)

    def wdiv(X):
        # sum_d sum_c D_d[c, r_d(a)] * gpvol(b) * sum_i He(i, d, b) X_i(b)
        G = gp[..., None] * np.einsum("...id,...i->...d", Hm, X)
        ox = np.einsum("cr,ekjc->ekjr", D[0], G[..., 0])
        oy = np.einsum("cr,ekcI->ekrI", D[1], G[..., 1])
        oz = np.einsum("cr,ecjI->erjI", D[2], G[..., 2])
        return ox + oy + oz

    nu_e = me / r
    kappa = muf * Cp / Pr + me * Cp / Pr + Cp * r * ms / 0.9
    Dm = nu_e * wdiv(gR)
    De = wdiv(tauU) + kappa * wdiv(gT)
    Dmom = [wdiv(tau[..., m, :]) for m in range(3)]
    out_m = np.zeros(npoin)
    out_mom = np.zeros((3, npoin))
    out_e = np.zeros(npoin)
    np.add.at(out_m, nodes, Dm)
    for c in range(3):
        np.add.at(out_mom[c], nodes, Dmom[c])
    np.add.at(out_e, nodes, De)
    return out_m, out_mom.reshape(-1), out_e


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    if nb == 0.0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def lumped_mass(geom, nelem, npoin, n):
    M = np.zeros(npoin)
    nodes = geom["connec"].reshape(n, nelem).T - 1
    np.add.at(M, nodes, geom["gpvol"].astype(np.float64).reshape(nelem, n))
    return M


# ---------------------------------------------------------------------------
# Linear tetrahedra (elem_convec.f90:839-948, elem_diffu.f90:199-317), whole
# mesh at once with einsum; arrays as in the C oracle (flattened Fortran).
# ---------------------------------------------------------------------------

def _tet_gather(nelem, npoin, connec, Ngp, dNgp, He, gpvol):
    con = np.asarray(connec).reshape(4, nelem).T - 1                   # [e, a]
    H = np.asarray(He, np.float64).reshape(nelem, 4, 3, 3)             # [e, g, j, i] = He(i,j,g,e)
    dN = np.asarray(dNgp, np.float64).reshape(4, 4, 3)                 # [g, a, j]
    gpcar = np.einsum("egji,gaj->egai", H, dN)                         # [e, g, a, i]
    gv = np.asarray(gpvol, np.float64).reshape(nelem, 4)               # [e, g]
    Nf = np.asarray(Ngp, np.float64).reshape(4, 4)                     # Nf[c, r] = Ngp(r, c)
    return con, gpcar, gv, Nf


def _vec(x, npoin, con):
    return np.asarray(x, np.float64).reshape(3, npoin).T[con]           # [e, a, i]


def _tet_scatter(con, npoin, Rm, Rq, Re):
    Rmass = np.zeros(npoin)
    Rener = np.zeros(npoin)
    Rmom = np.zeros((3, npoin))
    np.add.at(Rmass, con, Rm)
    np.add.at(Rener, con, Re)
    for i in range(3):
        np.add.at(Rmom[i], con, Rq[..., i])
    return Rmass, Rmom.reshape(-1), Rener


def fem_convec(nelem, npoin, connec, Ngp, dNgp, He, gpvol, u, q, rho, pr, E):
    con, gc, gv, Nf = _tet_gather(nelem, npoin, connec, Ngp, dNgp, He, gpvol)
    U, Qv = _vec(u, npoin, con), _vec(q, npoin, con)
    r = np.asarray(rho, np.float64)[con]
    p = np.asarray(pr, np.float64)[con]
    Ep = np.asarray(E, np.float64)[con] + p
    divQ = np.einsum("egai,eai->eg", gc, Qv)
    divFe = np.einsum("egai,ea,eai->eg", gc, Ep, U)
    gR = np.einsum("egai,ea->egi", gc, r)
    gE = np.einsum("egai,ea->egi", gc, Ep)
    gP = np.einsum("egai,ea->egi", gc, p)
    gU = np.einsum("egaj,eai->egij", gc, U)                            # d u_i / d x_j
    divF = np.einsum("egaj,eai,eaj->egi", gc, Qv, U)
    divU = np.einsum("egii->eg", gU)
    w = gv[:, :, None] * Nf.T[None, :, :] * 0.5                       # [e, g, a]: Ngp(igaus, inode)
    aux1 = np.einsum("egi,eai->ega", gR, U)
    aux2 = np.einsum("egi,eai->ega", gE, U)
    Rm = np.einsum("ega,ega->ea", w, divQ[:, :, None] + r[:, None, :] * divU[:, :, None] + aux1)
    Re = np.einsum("ega,ega->ea", w, divFe[:, :, None] + Ep[:, None, :] * divU[:, :, None] + aux2)
    aux3 = np.einsum("egij,eaj->egai", gU, Qv)
    aux4 = np.einsum("eai,eaj,egj->egai", U, U, gR)
    mom = divF[:, :, None, :] + Qv[:, None, :, :] * divU[:, :, None, None] + aux3 + aux4 + gP[:, :, None, :]
    Rq = np.einsum("ega,egai->eai", w, mom)
    return _tet_scatter(con, npoin, Rm, Rq, Re)


def fem_diffu(nelem, npoin, connec, Ngp, dNgp, He, gpvol, Cp, Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs):
    con, gc, gv, Nf = _tet_gather(nelem, npoin, connec, Ngp, dNgp, He, gpvol)
    N2 = Nf                                                            # N2[g, a] = Ngp(inode=a, igaus=g)
    U = _vec(u, npoin, con)
    r = np.asarray(rho, np.float64)[con]
    T = np.asarray(Tem, np.float64)[con]
    mf = np.asarray(mu_fluid, np.float64)[con]
    me = np.asarray(mu_e, np.float64).reshape(4, nelem).T
    ms = np.asarray(mu_sgs, np.float64).reshape(4, nelem).T
    aRho = np.einsum("ga,ea->eg", N2, r)
    aNu = np.einsum("ga,ea->eg", N2, me) / aRho
    aMu = np.einsum("ga,ega->eg", N2, mf[:, None, :] + aRho[:, :, None] * ms[:, None, :] + me[:, None, :])
    aKap = np.einsum("ga,ega->eg", N2, mf[:, None, :] * (Cp / Pr) + me[:, None, :] / 0.4
                     + aRho[:, :, None] * ms[:, None, :] / 0.9)
    gR = np.einsum("egai,ea->egi", gc, r)
    gT = np.einsum("egai,ea->egi", gc, T)
    gU = np.einsum("egai,eaj->egij", gc, U)                            # gradU(i,j) = d u_j / d x_i
    divU = np.einsum("egii->eg", gU)
    tau = gU + np.swapaxes(gU, 2, 3) - (2.0 / 3.0) * divU[:, :, None, None] * np.eye(3)
    aU = np.einsum("ga,eaj->egj", N2, U)
    tauU = np.einsum("egij,egj->egi", tau, aU)
    Rm = np.einsum("eg,egai,egi->ea", gv * aNu, gc, gR)
    Re = np.einsum("eg,egai,egi->ea", gv, gc, aMu[:, :, None] * tauU + aKap[:, :, None] * gT)
    Rq = np.einsum("eg,egaj,egij->eai", gv * aMu, gc, tau)
    return _tet_scatter(con, npoin, Rm, Rq, Re)


def tet_mesh_shared(n, jitter=0.0, seed=0):
    """Shared-node tet mesh of an n^3 grid of cubes of the unit cube: six
    tetrahedra per cube around its main diagonal (Kuhn), interior vertices
    jittered.  Returns (connec[a*E+e] 1-based int32, coord[d*npoin+p] float32, nelem, npoin)."""
    m = n + 1
    g = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3).astype(np.float64) / n
    rng = np.random.default_rng(seed)
    inner = np.all((g > 0) & (g < 1), axis=1)
    g[inner] += jitter / n * rng.uniform(-1, 1, (int(inner.sum()), 3))
    vid = lambda i, j, k: (i * m + j) * m + k
    tets = []
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    for i in range(n):
        for j in range(n):
            for k in range(n):
                for pm in perms:
                    c = [i, j, k]
                    t = [vid(*c)]
                    for ax in pm:
                        c = list(c)
                        c[ax] += 1
                        t.append(vid(*c))
                    if pm in ((0, 2, 1), (1, 0, 2), (2, 1, 0)):  # odd permutation: positive orientation
                        t[1], t[2] = t[2], t[1]
                    tets.append(t)
    tets = np.array(tets, np.int64)
    nelem, npoin = len(tets), m ** 3
    connec = (tets.T.reshape(-1) + 1).astype(np.int32)
    coord = g.T.reshape(-1).astype(np.float32)
    return connec, coord, nelem, npoin
