"""The oracle's restatement of the lumped mass and the RK4 step (oracle.lumped_mass,
oracle.rk4_step), on a mesh and fields built by the oracle alone (CPU).

Checks: the lumped mass of the unit cube sums to its volume and is positive; a uniform flow is a
steady state of the step; and the step's local error falls as dt^5 (fourth order): one step of dt
against two of dt/2 differ by C dt^5, so halving dt divides the difference by about 32.
"""
import numpy as np

from oracle import oracle as O


def _case(P=2, nx=2, jitter=0.05, seed=3):
    t64 = O.element_tables(P, np.float64)
    t32 = O.element_tables(P, np.float32)
    connec, coord, nelem, npoin = O.structured_mesh(P, nx, t32, jitter, seed)
    He, gpvol = O.elem_jacobian(P, nelem, npoin, connec, coord, t64["dNgp"], t64["wgp"], np.float64)
    geom = dict(t64, connec=connec, He=He, gpvol=gpvol)
    f = O.fields_recipe(0, 4, seed, npoin, coord)
    n = (P + 1) ** 3
    rng = np.random.default_rng(seed)
    mu_e = 1e-3 * rng.random(nelem * n)
    mu_sgs = 5e-4 * rng.random(nelem * n)
    return P, nelem, npoin, geom, f, mu_e, mu_sgs


def _step(case, dt, U, Ml):
    P, nelem, npoin, geom, f, mu_e, mu_sgs = case
    return O.rk4_step(P, nelem, npoin, geom, 1004.5, 0.71, 1.4, 287.0, Ml, f["mu_fluid"], mu_e, mu_sgs, dt, *U,
                      dtype=np.float64)


def _state(case):
    f = case[4]
    rho = f["rho"].astype(np.float64)
    return [rho, f["q"].astype(np.float64), rho * f["E"].astype(np.float64)]


def test_lumped_mass_volume():
    P, nelem, npoin, geom, *_ = _case()
    Ml = O.lumped_mass(P, nelem, npoin, geom["connec"], geom["gpvol"])
    assert np.all(Ml > 0)
    assert abs(Ml.sum() - 1.0) < 1e-12


def test_uniform_flow_is_steady():
    case = _case()
    P, nelem, npoin, geom, *_ = case
    Ml = O.lumped_mass(P, nelem, npoin, geom["connec"], geom["gpvol"])
    u = np.array([0.3, -0.1, 0.2])
    U = [np.full(npoin, 1.2), np.repeat(1.2 * u, npoin), np.full(npoin, 2.5 + 0.6 * (u * u).sum())]
    U1 = _step(case, 1e-2, U, Ml)
    for a, b in zip(U1, U):
        assert np.max(np.abs(a - b)) <= 1e-11 * np.max(np.abs(b))


def test_fourth_order_local_error():
    case = _case()
    P, nelem, npoin, geom, *_ = case
    Ml = O.lumped_mass(P, nelem, npoin, geom["connec"], geom["gpvol"])
    U = _state(case)

    def defect(dt):
        one = _step(case, dt, U, Ml)
        two = _step(case, dt / 2, _step(case, dt / 2, U, Ml), Ml)
        return np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(one, two)))

    d1, d2 = defect(2e-2), defect(1e-2)
    ratio = d1 / d2
    print("RK4 local error ratio %.1f (%.3e / %.3e)" % (ratio, d1, d2))
    assert 20.0 < ratio < 45.0
