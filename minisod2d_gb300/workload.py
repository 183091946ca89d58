"""Named workloads (mesh + seeded fields) and their device residency.

The five workloads of the project's scope:
  plain_16      16^3 hexes, porder 4, affine, smooth fields (8 modes)         -- CPU-runnable parity case
  plain_64      64^3 hexes, porder 4, +-5% jitter, smooth fields (8 modes)    -- the throughput workload
  plain_32      32^3 hexes, same recipe (profiling size: 0.3 GB per call, > L2)
  mixed_p7      32^3 hexes, porder 7, +-5% jitter, smooth fields (16 modes)
  learned_48    48^3 hexes, porder 4, affine, shock-like fields (8 modes)
  combined_96   96^3 hexes, porder 5, +-5% jitter, shock-like fields (8 modes)
All fields are FP32 with seed 0 unless stated; mu_fluid = 1.8e-5,
mu_e = mu_sgs = 0, Cp = 1004.5, Pr = 0.71.
"""
from dataclasses import dataclass

import numpy as np

from . import capi, fem


@dataclass(frozen=True)
class Config:
    name: str
    porder: int
    nx: int
    jitter: float
    kind: int
    nmodes: int
    seed: int = 0
    Cp: float = 1004.5
    Pr: float = 0.71

    @property
    def nelem(self):
        return self.nx ** 3

    @property
    def npoin(self):
        return (self.nx * self.porder + 1) ** 3

    @property
    def nnode(self):
        return (self.porder + 1) ** 3


CONFIGS = {
    "plain_16": Config("plain_16", 4, 16, 0.0, capi.MSOD_FIELDS_SMOOTH, 8),
    "plain_64": Config("plain_64", 4, 64, 0.05, capi.MSOD_FIELDS_SMOOTH, 8),
    "plain_32": Config("plain_32", 4, 32, 0.05, capi.MSOD_FIELDS_SMOOTH, 8),
    "mixed_p7": Config("mixed_p7", 7, 32, 0.05, capi.MSOD_FIELDS_SMOOTH, 16),
    "learned_48": Config("learned_48", 4, 48, 0.0, capi.MSOD_FIELDS_SHOCK, 8),
    "combined_96": Config("combined_96", 5, 96, 0.05, capi.MSOD_FIELDS_SHOCK, 8),
}


def custom(porder, nx, jitter=0.0, kind=capi.MSOD_FIELDS_SMOOTH, nmodes=8, seed=0):
    return Config("custom_p%d_n%d" % (porder, nx), porder, nx, jitter, kind, nmodes, seed)


class HostCase:
    """Host arrays of a workload: element tables, mesh, node fields (numpy)."""

    def __init__(self, cfg, dtype=np.float32):
        self.cfg = cfg
        self.tables = fem.element_tables(cfg.porder, np.float32)
        self.connec, self.coord, self.nelem, self.npoin = fem.structured_mesh(
            cfg.porder, cfg.nx, cfg.nx, cfg.nx, self.tables, cfg.jitter, cfg.seed)
        self.fields = fem.fields_recipe(cfg.kind, cfg.nmodes, cfg.seed, self.npoin, self.coord)
        n = cfg.nnode
        self.mu_e = np.zeros(self.nelem * n, np.float32)
        self.mu_sgs = np.zeros(self.nelem * n, np.float32)

    def with_seed(self, seed):
        """The same mesh with the fields of another seed."""
        import copy

        other = copy.copy(self)
        other.cfg = Config(self.cfg.name, self.cfg.porder, self.cfg.nx, self.cfg.jitter, self.cfg.kind,
                           self.cfg.nmodes, int(seed), self.cfg.Cp, self.cfg.Pr)
        other.fields = fem.fields_recipe(self.cfg.kind, self.cfg.nmodes, int(seed), self.npoin, self.coord)
        return other


class DeviceCase:
    """A workload resident on the GPU as torch tensors, metric built on the device."""

    def set_fields(self, host):
        """Upload the node fields of another HostCase on the same mesh."""
        import torch

        self.host = host
        self.cfg = host.cfg
        for k, v in host.fields.items():
            getattr(self, k).copy_(torch.from_numpy(v))

    def __init__(self, host, device="cuda", dtype=None):
        import torch

        dtype = dtype or torch.float32
        self.host = host
        self.cfg = host.cfg
        self.dtype = dtype
        self.nelem, self.npoin = host.nelem, host.npoin
        t = host.tables
        dev = torch.device(device)

        def up(a, dt=None):
            return torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)

        self.connec = up(host.connec)
        self.invAtoIJK = up(t["invAtoIJK"])
        self.AtoI, self.AtoJ, self.AtoK = up(t["AtoI"]), up(t["AtoJ"]), up(t["AtoK"])
        if dtype == torch.float64:
            t64 = fem.element_tables(self.cfg.porder, np.float64)
            self.dlxigp_ip = up(t64["dlxigp_ip"])
            dN, w = up(t64["dNgp"]), up(t64["wgp"])
        else:
            self.dlxigp_ip = up(t["dlxigp_ip"])
            dN, w = up(t["dNgp"]), up(t["wgp"])
        coord = up(host.coord, dtype)
        n = self.cfg.nnode
        self.He = torch.empty(9 * self.nelem * n, dtype=dtype, device=dev)
        self.gpvol = torch.empty(self.nelem * n, dtype=dtype, device=dev)
        from . import kernels

        kernels.elem_jacobian(self.cfg.porder, self.nelem, self.npoin, self.connec, coord, dN, w, self.gpvol, self.He)
        del coord
        f = host.fields
        for k in ("rho", "u", "q", "pr", "E", "Tem", "mu_fluid"):
            setattr(self, k, up(f[k], dtype))
        self.mu_e = up(host.mu_e, dtype)
        self.mu_sgs = up(host.mu_sgs, dtype)
        self.Rmass = torch.empty(self.npoin, dtype=dtype, device=dev)
        self.Rmom = torch.empty(3 * self.npoin, dtype=dtype, device=dev)
        self.Rener = torch.empty(self.npoin, dtype=dtype, device=dev)
        self.Dmass = torch.empty_like(self.Rmass)
        self.Dmom = torch.empty_like(self.Rmom)
        self.Dener = torch.empty_like(self.Rener)

    def geometry(self):
        return (self.nelem, self.npoin, self.connec, None, None, self.He, self.gpvol, self.dlxigp_ip, None,
                self.invAtoIJK, self.AtoI, self.AtoJ, self.AtoK)

    def convec(self, split=False, stream=None):
        from . import kernels

        kernels.full_convec_ijk(*self.geometry(), self.u, self.q, self.rho, self.pr, self.E, self.Rmass, self.Rmom,
                                self.Rener, stream=stream, split=split)
        return self.Rmass, self.Rmom, self.Rener

    def convec_mixed(self, precision="fp16", out=None, stream=None):
        """Mixed-precision convection into FP64 residuals (allocated unless ``out`` is given)."""
        import torch

        from . import kernels

        if out is None:
            dev = self.He.device
            out = (torch.empty(self.npoin, dtype=torch.float64, device=dev),
                   torch.empty(3 * self.npoin, dtype=torch.float64, device=dev),
                   torch.empty(self.npoin, dtype=torch.float64, device=dev))
        g = self.geometry()
        kernels.full_convec_ijk_mixed(g[0], g[1], g[2], g[5], g[6], g[7], *g[9:], self.u, self.q, self.rho, self.pr,
                                      self.E, *out, precision=precision, stream=stream)
        return out

    def diffu_mixed(self, precision="fp16", mu_e=None, nu_elem=None, out=None, stream=None):
        """Mixed-precision diffusion into FP64 residuals (allocated unless ``out`` is given)."""
        import torch

        from . import kernels

        if out is None:
            dev = self.He.device
            out = (torch.empty(self.npoin, dtype=torch.float64, device=dev),
                   torch.empty(3 * self.npoin, dtype=torch.float64, device=dev),
                   torch.empty(self.npoin, dtype=torch.float64, device=dev))
        g = self.geometry()
        kernels.full_diffusion_ijk_mixed(g[0], g[1], g[2], g[5], g[6], g[7], *g[9:], self.cfg.Cp, self.cfg.Pr,
                                         self.rho, self.u, self.Tem, self.mu_fluid,
                                         self.mu_e if mu_e is None else mu_e, self.mu_sgs, *out,
                                         precision=precision, nu_elem=nu_elem, stream=stream)
        return out

    def diffu(self, stream=None):
        from . import kernels

        kernels.full_diffusion_ijk(*self.geometry(), self.cfg.Cp, self.cfg.Pr, self.rho, self.u, self.Tem,
                                   self.mu_fluid, self.mu_e, self.mu_sgs, self.Dmass, self.Dmom, self.Dener,
                                   stream=stream)
        return self.Dmass, self.Dmom, self.Dener

    def convec_diffu(self, stream=None):
        """Both residuals in one call (msod_convec_diffusion_ijk) into the same arrays as convec and diffu."""
        from . import kernels

        kernels.full_convec_diffusion_ijk(*self.geometry(), self.cfg.Cp, self.cfg.Pr, self.u, self.q, self.rho,
                                          self.pr, self.E, self.Tem, self.mu_fluid, self.mu_e, self.mu_sgs,
                                          self.Rmass, self.Rmom, self.Rener, self.Dmass, self.Dmom, self.Dener,
                                          stream=stream)
        return (self.Rmass, self.Rmom, self.Rener), (self.Dmass, self.Dmom, self.Dener)


class TetCase:
    """The reference driver's TET04 data (main.f90:365-407) on the GPU.

    Disconnected unit tetrahedra (gen_tet_mesh): npoin_t = 4 nelem_t nodes,
    taken as the first multiple of 4 of a hex workload's nodes, whose node
    fields the tet kernels read (the driver passes the same u, q, rho, pr, E,
    Tem, mu_fluid to its hex and tet kernels); mu_e = mu_sgs = 1
    (main.f90:402-406); metric by tet_jacobian on the device.
    """

    def __init__(self, host, device="cuda", dtype=None):
        import torch

        from . import kernels

        dtype = dtype or torch.float32
        np_dt = np.float32 if dtype == torch.float32 else np.float64
        dev = torch.device(device)
        self.dtype = dtype
        self.npoin = (host.npoin // 4) * 4
        self.nelem = self.npoin // 4
        t = fem.tet_element_tables(np_dt)
        connec, coord, _ = fem.tet_mesh_disconnected(self.nelem)

        def up(a, dt=None):
            return torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)

        self.connec = up(connec)
        self.Ngp, self.dNgp = up(t["Ngp"]), up(t["dNgp"])
        c = up(coord, dtype)
        self.He = torch.empty(36 * self.nelem, dtype=dtype, device=dev)
        self.gpvol = torch.empty(4 * self.nelem, dtype=dtype, device=dev)
        kernels.tet_jacobian(self.nelem, self.npoin, self.connec, c, self.dNgp, up(t["wgp"]), self.gpvol, self.He)
        del c
        f, n, m = host.fields, self.npoin, host.npoin
        for k in ("rho", "pr", "E", "Tem", "mu_fluid"):
            setattr(self, k, up(f[k][:n], dtype))
        for k in ("u", "q"):
            setattr(self, k, up(f[k].reshape(3, m)[:, :n].reshape(-1), dtype))
        self.mu_e = torch.ones(4 * self.nelem, dtype=dtype, device=dev)
        self.mu_sgs = torch.ones(4 * self.nelem, dtype=dtype, device=dev)
        self.Cp, self.Pr = 1.0, 1.0  # main.f90:412-413
        self.R = tuple(torch.empty(k * n, dtype=dtype, device=dev) for k in (1, 3, 1))
        self.D = tuple(torch.empty(k * n, dtype=dtype, device=dev) for k in (1, 3, 1))

    def convec(self, stream=None):
        from . import kernels

        kernels.fem_convec(self.nelem, self.npoin, self.connec, self.Ngp, self.dNgp, self.He, self.gpvol, self.u,
                           self.q, self.rho, self.pr, self.E, *self.R, stream=stream)
        return self.R

    def diffu(self, stream=None):
        from . import kernels

        kernels.fem_diffu(self.nelem, self.npoin, self.connec, self.Ngp, self.dNgp, self.He, self.gpvol, self.Cp,
                          self.Pr, self.rho, self.u, self.Tem, self.mu_fluid, self.mu_e, self.mu_sgs, *self.D,
                          stream=stream)
        return self.D

    # Algorithmic bytes per element: connec 16, He 144, gpvol 16, node fields
    # (convection: u, q, rho, pr, E = 9 values; diffusion: rho, u, Tem, mu_fluid
    # = 6 values and mu_e, mu_sgs 2 x 4 per element) and 5 residuals per node,
    # every value read or written once.
    def algorithmic_bytes(self, which):
        reals = 36 + 4 + (4 * 9 if which == "convec" else 4 * 6 + 2 * 4) + 4 * 5
        return self.nelem * (4 * 4 + reals * self.dtype.itemsize)
