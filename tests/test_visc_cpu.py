"""CPU checks of the viscosity estimators' references (no GPU)."""
import numpy as np
import pytest

from minisod2d_gb300 import workload
from oracle import oracle as O
from tests import mlp_ref, refimpl


def _case(P=4, nx=3, seed=1, kind=1):
    cfg = workload.Config("t", P, nx, 0.05, kind, 8, seed)
    h = workload.HostCase(cfg)
    t = O.element_tables(P, np.float64)
    He, gp = O.elem_jacobian(P, h.nelem, h.npoin, h.connec, h.coord.astype(np.float64), t["dNgp"], t["wgp"], np.float64)
    return h, dict(t, connec=h.connec, He=He, gpvol=gp)


def _numpy_estimator(t, geom, nelem, npoin, rho, u, pr, gamma=1.4, ce=0.1, cmax=0.5):
    inv, D, nodes, Hm, gp = refimpl._gather(geom, nelem, t)
    r = np.asarray(rho, np.float64)[nodes]
    p = np.asarray(pr, np.float64)[nodes]
    U = np.stack([np.asarray(u[c * npoin:(c + 1) * npoin], np.float64) for c in range(3)], -1)[nodes]
    eta = r / (gamma - 1) * (np.log(p) - gamma * np.log(r))
    ge = refimpl._grad(Hm, refimpl._iso(D, eta))
    divf = sum(refimpl._grad(Hm, refimpl._iso(D, eta * U[..., i]))[..., i] for i in range(3))
    divu = sum(refimpl._grad(Hm, refimpl._iso(D, U[..., i]))[..., i] for i in range(3))
    R = np.abs(divf - eta * divu - (U * ge).sum(-1))
    eall = np.asarray(rho, np.float64) / (gamma - 1) * (np.log(np.asarray(pr, np.float64)) - gamma * np.log(np.asarray(rho, np.float64)))
    neta = max(eall.max() - eall.mean(), eall.mean() - eall.min())
    spd = np.linalg.norm(U, axis=-1) + np.sqrt(gamma * p / r)
    h = np.cbrt(gp.reshape(nelem, -1).sum(1)) / t["P"]
    numax = cmax * h * spd.reshape(nelem, -1).max(1)
    nuE = ce * h * h * R.reshape(nelem, -1).max(1) / neta
    return np.minimum(numax, nuE), numax


def test_oracle_estimator_matches_numpy():
    h, geom = _case()
    f = h.fields
    mu, nu, numax = O.entropy_viscosity(4, h.nelem, h.npoin, geom, f["rho"], f["u"], f["pr"])
    nu2, numax2 = _numpy_estimator(geom, geom, h.nelem, h.npoin, f["rho"], f["u"], f["pr"])
    assert np.allclose(numax, numax2, rtol=1e-12)
    assert np.allclose(nu, nu2, rtol=1e-9)
    con = np.asarray(h.connec).reshape(-1, h.nelem)
    assert np.allclose(mu.reshape(-1, h.nelem), f["rho"][con - 1] * nu[None, :], rtol=1e-6)


def test_estimator_is_small_for_resolved_fields():
    """On smooth, resolved fields the entropy residual (a product-rule defect) is
    far below the first-order viscosity; across the shock-like front it is not."""
    hs, gs = _case(kind=0)
    f = hs.fields
    _, nu_s, numax_s = O.entropy_viscosity(4, hs.nelem, hs.npoin, gs, f["rho"], f["u"], f["pr"])
    hk, gk = _case(kind=1)
    f = hk.fields
    _, nu_k, numax_k = O.entropy_viscosity(4, hk.nelem, hk.npoin, gk, f["rho"], f["u"], f["pr"])
    assert (nu_s / numax_s).max() < (nu_k / numax_k).max()


def test_numpy_mlp_gradient_finite_differences():
    rng = np.random.default_rng(0)
    w = rng.normal(0, 0.3, mlp_ref.NPARAMS)
    norm = np.concatenate([rng.normal(0, 1, 12), rng.uniform(0.5, 2, 12), -np.ones(12) * 1e30, np.ones(12) * 1e30])
    x = rng.normal(0, 1, (16, 12))
    t = rng.uniform(0, 1, 16)
    for wt in (None, rng.uniform(0.1, 5.0, 16)):  # plain and per-sample weighted loss
        g = mlp_ref.gradient(w, norm, x, t, wt)
        for k in rng.choice(mlp_ref.NPARAMS, 40, replace=False):
            e = np.zeros_like(w)
            e[k] = 1e-6
            fd = (mlp_ref.loss(w + e, norm, x, t, wt) - mlp_ref.loss(w - e, norm, x, t, wt)) / 2e-6
            assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(g[k])


def test_numpy_features_are_finite():
    h, geom = _case()
    f = h.fields
    F, numax = mlp_ref.features(geom, geom, h.nelem, h.npoin, f["rho"], f["u"], f["pr"])
    assert np.all(np.isfinite(F)) and np.all(numax > 0)
    _, _, numax_o = O.entropy_viscosity(4, h.nelem, h.npoin, geom, f["rho"], f["u"], f["pr"])
    assert np.allclose(numax, numax_o, rtol=1e-12)


@pytest.mark.parametrize("name", ["learned_48", "combined_96"])
def test_shipped_weight_file_format(name):
    """The committed networks: magic, sizes and CRC-32 of the weight files."""
    import struct
    import zlib

    from minisod2d_gb300 import learn

    b = open(learn.shipped_weights(name), "rb").read()
    assert b[:8] == b"MSODMLP1"
    ver, nin, nh, npar = struct.unpack("<4i", b[8:24])
    assert (ver, nin, nh, npar) == (1, 12, 32, mlp_ref.NPARAMS)
    assert len(b) == 24 + 4 * 48 + 2 * npar + 4
    assert zlib.crc32(b[:-4]) == struct.unpack("<I", b[-4:])[0]
    norm = np.frombuffer(b[24:24 + 192], np.float32)
    assert np.all(norm[24:36] <= norm[36:48])  # training ranges
    w = np.frombuffer(b[216:216 + 2 * npar], np.float16)
    assert np.all(np.isfinite(w))
