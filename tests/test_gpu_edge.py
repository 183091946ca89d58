"""Edge cases of the hex kernels on the GPU: one element, nodes that no element
references, and equivariance under renumbering (a random node relabelling and
element shuffle permute the residuals and change nothing else)."""
import numpy as np
import pytest

from minisod2d_gb300 import kernels, workload
from oracle import oracle as O
from tests import refimpl

pytestmark = pytest.mark.gpu


class Arrays:
    """Host arrays of a case that the test may renumber, and calls on them."""

    def __init__(self, host, dev):
        self.P = host.cfg.porder
        self.n = host.cfg.nnode
        self.nelem, self.npoin = host.nelem, host.npoin
        self.t = host.tables
        self.connec = host.connec.copy()
        self.He = dev.He.cpu().numpy().copy()
        self.gpvol = dev.gpvol.cpu().numpy().copy()
        self.f = {k: v.copy() for k, v in host.fields.items()}
        rng = np.random.default_rng(9)
        self.mu_e = (1e-3 * rng.random(self.nelem * self.n)).astype(np.float32)
        self.mu_sgs = (1e-3 * rng.random(self.nelem * self.n)).astype(np.float32)
        self.Cp, self.Pr = host.cfg.Cp, host.cfg.Pr

    def run(self, cuda):
        import torch

        up = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=cuda)
        t = self.t
        geo = (self.nelem, self.npoin, up(self.connec), None, None, up(self.He), up(self.gpvol), up(t["dlxigp_ip"]),
               None, up(t["invAtoIJK"]), up(t["AtoI"]), up(t["AtoJ"]), up(t["AtoK"]))
        f = {k: up(v) for k, v in self.f.items()}
        R = [torch.empty(k * self.npoin, device=cuda) for k in (1, 3, 1)]
        D = [torch.empty(k * self.npoin, device=cuda) for k in (1, 3, 1)]
        kernels.full_convec_ijk(*geo, f["u"], f["q"], f["rho"], f["pr"], f["E"], *R)
        kernels.full_diffusion_ijk(*geo, self.Cp, self.Pr, f["rho"], f["u"], f["Tem"], f["mu_fluid"],
                                   up(self.mu_e), up(self.mu_sgs), *D)
        return [x.cpu().numpy().astype(np.float64) for x in R + D]


def _case(cuda, P, nx, seed=0):
    host = workload.HostCase(workload.Config("edge", P, nx, 0.05, 1, 8, seed))
    return Arrays(host, workload.DeviceCase(host, device=cuda))


@pytest.mark.parametrize("P", [1, 4, 7])
def test_single_element(cuda, P):
    c = _case(cuda, P, 1, seed=P)
    got = c.run(cuda)
    geom = dict(c.t, connec=c.connec, He=c.He, gpvol=c.gpvol)
    f = c.f
    rc = O.full_convec_ijk(P, 1, c.npoin, geom, f["u"], f["q"], f["rho"], f["pr"], f["E"], dtype=np.float64)
    rd = O.full_diffusion_ijk(P, 1, c.npoin, geom, c.Cp, c.Pr, f["rho"], f["u"], f["Tem"], f["mu_fluid"], c.mu_e,
                              c.mu_sgs, dtype=np.float64)
    for g, r in zip(got, list(rc) + list(rd)):
        assert refimpl.rel_l2(g, r) < 1e-5


def test_unreferenced_nodes_get_zero(cuda):
    c = _case(cuda, 4, 2)
    base = c.run(cuda)
    extra, np0 = 77, c.npoin
    rng = np.random.default_rng(1)
    for k, v in list(c.f.items()):
        comps = v.size // np0
        parts = [np.concatenate([v[i * np0:(i + 1) * np0], (1.0 + rng.random(extra)).astype(np.float32)])
                 for i in range(comps)]
        c.f[k] = np.concatenate(parts)
    c.npoin = np0 + extra
    got = c.run(cuda)
    for g, b in zip(got, base):
        comps = b.size // np0
        g2 = g.reshape(comps, c.npoin)
        assert np.all(g2[:, np0:] == 0.0)
        assert refimpl.rel_l2(g2[:, :np0].reshape(-1), b) < 1e-6


def test_renumbering_equivariance(cuda):
    c = _case(cuda, 4, 3, seed=4)
    base = c.run(cuda)
    rng = np.random.default_rng(5)
    n, E, npn = c.n, c.nelem, c.npoin
    perm = rng.permutation(npn)            # new id of old node p is perm[p]
    eperm = rng.permutation(E)             # new element k is old element eperm[k]
    con = c.connec.reshape(n, E)
    c.connec = (perm[con[:, eperm] - 1] + 1).astype(np.int32).reshape(-1)
    c.He = c.He.reshape(E, -1)[eperm].reshape(-1)
    c.gpvol = c.gpvol.reshape(E, -1)[eperm].reshape(-1)
    c.mu_e = c.mu_e.reshape(n, E)[:, eperm].reshape(-1)
    c.mu_sgs = c.mu_sgs.reshape(n, E)[:, eperm].reshape(-1)
    inv = np.argsort(perm)                 # old node of new id
    for k, v in list(c.f.items()):
        comps = v.size // npn
        c.f[k] = v.reshape(comps, npn)[:, inv].reshape(-1)
    got = c.run(cuda)
    for g, b in zip(got, base):
        comps = b.size // npn
        back = g.reshape(comps, npn)[:, perm].reshape(-1)   # new results at the old node ids
        assert refimpl.rel_l2(back, b) < 1e-6
