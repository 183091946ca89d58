"""Time integration around the two residual calls: the lumped mass matrix and the
classical RK4 step of dU/dt = -Ml^-1 (R_conv + R_diff), U = (rho, q = rho u, rhoE)
(msod_lumped_mass, msod_rk4_step; the reference names both, flag_rk_order = 4 and
flag_solver_type = 1 in mod_numerical_params.f90:8,20, without containing them).
"""
import ctypes as C

from . import capi

GAMMA = 1.4
RGAS = 287.0  # main.f90:52


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(stream):
    if stream is not None:
        return stream
    import torch

    return torch.cuda.current_stream().cuda_stream


def lumped_mass(dev, Ml=None, stream=None):
    """Ml(p) = sum of gpvol(e, g) over the element points g at node p (device tensor, npoin)."""
    import torch

    Ml = Ml if Ml is not None else torch.empty(dev.npoin, dtype=torch.float32, device=dev.He.device)
    capi.call("msod_lumped_mass", dev.cfg.porder, dev.nelem, dev.npoin, _p(dev.connec), _p(dev.gpvol), _p(Ml),
              _stream(stream))
    return Ml


def workspace(dev):
    """A device workspace of the size msod_rk4_step needs."""
    import torch

    n = C.c_size_t(0)
    capi.call("msod_rk4_workspace_bytes", dev.npoin, C.byref(n))
    return torch.empty(n.value, dtype=torch.uint8, device=dev.He.device)


def rk4_step(dev, Ml, dt, rho, q, rhoE, ws, gamma=GAMMA, Rgas=RGAS, mu_e=None, mu_sgs=None, stream=None):
    """One RK4 step on the state (rho, q, rhoE), updated in place; mu_fluid, mu_e and mu_sgs from the
    case unless given."""
    capi.call("msod_rk4_step", dev.cfg.porder, dev.nelem, dev.npoin, _p(dev.connec), _p(dev.He), _p(dev.gpvol),
              _p(dev.dlxigp_ip), _p(dev.invAtoIJK), _p(dev.AtoI), _p(dev.AtoJ), _p(dev.AtoK), float(dev.cfg.Cp),
              float(dev.cfg.Pr), float(gamma), float(Rgas), _p(Ml), _p(dev.mu_fluid),
              _p(dev.mu_e if mu_e is None else mu_e), _p(dev.mu_sgs if mu_sgs is None else mu_sgs), float(dt),
              _p(rho), _p(q), _p(rhoE), _p(ws), ws.numel(), _stream(stream))
    return rho, q, rhoE
