"""CPU reference of the per-element network (forward, backward, features) in numpy FP64.

Test infrastructure: the GPU network's forward pass, gradients and the
element features are checked against these restatements.
"""
import numpy as np

NIN, NH = 12, 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NIN
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH
NPARAMS = OFF_B3 + 1


def unpack(w):
    w = np.asarray(w, np.float64)
    return (w[OFF_W1:OFF_B1].reshape(NH, NIN), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(NH, NH), w[OFF_B2:OFF_W3],
            w[OFF_W3:OFF_B3], w[OFF_B3])


def fp16_round(w):
    return np.asarray(w, np.float32).astype(np.float16).astype(np.float64)


def sig(a):
    return 1.0 / (1.0 + np.exp(-a))


# Features stored as log(max(v, 0) + 1e-12); the others (mean Mach, max Mach,
# scaled divergence) stay linear.
LOG_FEATURES = [0, 1, 2, 6, 7, 8, 9, 10, 11]


def log_features(F):
    G = np.array(F, np.float64, copy=True)
    G[:, LOG_FEATURES] = np.log(np.maximum(G[:, LOG_FEATURES], 0.0) + 1e-12)
    return G


def raw_features(G):
    F = np.array(G, np.float64, copy=True)
    F[:, LOG_FEATURES] = np.exp(F[:, LOG_FEATURES]) - 1e-12
    return F


def s_from_y(y):
    """Training target of the network's output: decades below the bound."""
    return -np.log10(np.clip(np.asarray(y, np.float64), 1e-12, 1.0))


def y_from_s(s):
    return 10.0 ** (-np.asarray(s, np.float64))


def forward(w, norm, x):
    """x: (B, 12) features as stored; norm: 48 floats (mean, 1/std, min, max).
    Returns the softplus output s (y = 10^-s) and the activations."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    mean, inv_std = np.asarray(norm[:NIN], np.float64), np.asarray(norm[NIN:2 * NIN], np.float64)
    xh = (np.asarray(x, np.float64) - mean) * inv_std
    a1 = xh @ W1.T + b1
    h1 = a1 * sig(a1)
    a2 = h1 @ W2.T + b2
    h2 = a2 * sig(a2)
    z = h2 @ W3 + b3
    y = np.where(z > 20, z, np.log1p(np.exp(np.minimum(z, 20))))
    return y, (xh, a1, h1, a2, h2, z)


def gradient(w, norm, x, t, weight=None):
    """d/dw of mean(weight (s - s_from_y(t))^2) over the batch (weight 1 if None; flattened like the
    device layout)."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    y, (xh, a1, h1, a2, h2, z) = forward(w, norm, x)
    t = s_from_y(t)
    B = len(t)
    wt = np.ones(B) if weight is None else np.asarray(weight, np.float64)
    dz = 2.0 * wt * (y - t) / B * sig(z)
    gW3 = dz @ h2
    gb3 = dz.sum()
    dh2 = dz[:, None] * W3[None, :]
    da2 = dh2 * sig(a2) * (1 + a2 * (1 - sig(a2)))
    gW2 = da2.T @ h1
    gb2 = da2.sum(0)
    dh1 = da2 @ W2
    da1 = dh1 * sig(a1) * (1 + a1 * (1 - sig(a1)))
    gW1 = da1.T @ xh
    gb1 = da1.sum(0)
    g = np.zeros(NPARAMS)
    g[OFF_W1:OFF_B1] = gW1.ravel()
    g[OFF_B1:OFF_W2] = gb1
    g[OFF_W2:OFF_B2] = gW2.ravel()
    g[OFF_B2:OFF_W3] = gb2
    g[OFF_W3:OFF_B3] = gW3
    g[OFF_B3] = gb3
    return g


def loss(w, norm, x, t, weight=None):
    y, _ = forward(w, norm, x)
    wt = np.ones(len(t)) if weight is None else np.asarray(weight, np.float64)
    return float(np.mean(wt * (y - s_from_y(t)) ** 2))


def features(tables, geom, nelem, npoin, rho, u, pr, gamma=1.4, cmax=0.5):
    """The 12 element features and nu_max (FP64), restated from their definitions."""
    from tests import refimpl

    P = tables["P"]
    Q = P + 1
    n = Q ** 3
    inv, D = refimpl.lattice_maps(tables)
    perm = inv.reshape(-1)  # [(K*Q+J)*Q+I] -> gmsh node
    rho = np.asarray(rho, np.float64)
    pr = np.asarray(pr, np.float64)
    U = np.stack([np.asarray(u[c * npoin:(c + 1) * npoin], np.float64) for c in range(3)], -1)
    eta_all = rho / (gamma - 1) * (np.log(pr) - gamma * np.log(rho))
    mean = eta_all.mean()
    neta = max(eta_all.max() - mean, mean - eta_all.min())
    con = np.asarray(geom["connec"]).reshape(n, nelem) - 1
    He = np.asarray(geom["He"], np.float64).reshape(nelem, n, 3, 3)  # [e, g, j, i]
    gp = np.asarray(geom["gpvol"], np.float64).reshape(nelem, n)
    mnat = P // 2
    ms = 0 if mnat == 0 else (1 if mnat == P else mnat + 1)
    nat = [0, ms, 1]
    F = np.zeros((nelem, NIN))
    numax = np.zeros(nelem)
    for e in range(nelem):
        p = con[:, e]
        r, q, uu = rho[p], pr[p], U[p]
        c = np.sqrt(gamma * q / r)
        um = np.linalg.norm(uu, axis=1)
        s = (np.log(q) - gamma * np.log(r)) / (gamma - 1)
        eta = r * s
        h = np.cbrt(gp[e].sum()) / P
        node = lambda I, J, K: perm[(K * Q + J) * Q + I]
        d2r = d2e = defect = 0.0
        gi = np.zeros((3, 3))
        for d in range(3):
            idx = [node(*(nat[k] if dd == d else ms for dd in range(3))) for k in range(3)]
            rv, ev, uv = r[idx], eta[idx], uu[idx, d]
            d2r = max(d2r, abs(rv[0] - 2 * rv[1] + rv[2]))
            d2e = max(d2e, abs(ev[0] - 2 * ev[1] + ev[2]))
            A = ev[2] * uv[2] - ev[0] * uv[0]
            B = ev[1] * (uv[2] - uv[0]) + uv[1] * (ev[2] - ev[0])
            defect = max(defect, abs(A - B))
            line = [node(*(cc if dd == d else ms for dd in range(3))) for cc in range(Q)]
            for i in range(3):
                gi[i, d] = D[d, ms] @ uu[line, i]
        Hc = He[e, node(ms, ms, ms)]  # [j, i] = He(i, j)
        G = np.array([[sum(Hc[k, j] * gi[i, k] for k in range(3)) for j in range(3)] for i in range(3)])
        theta = np.trace(G)
        w = np.array([G[2, 1] - G[1, 2], G[0, 2] - G[2, 0], G[1, 0] - G[0, 1]])
        S = 0.5 * (G + G.T)
        sc = h / c.mean()
        F[e] = [(r.max() - r.min()) / r.mean(), (q.max() - q.min()) / q.mean(), s.max() - s.min(), um.mean() / c.mean(),
                (um / c).max(), theta * sc, np.linalg.norm(w) * sc, np.linalg.norm(S) * sc, d2r / r.mean(), d2e / neta,
                (eta.max() - eta.min()) / neta, defect / (neta * (um.mean() + c.mean()))]
        numax[e] = cmax * h * (um + c).max()
    return F, numax
