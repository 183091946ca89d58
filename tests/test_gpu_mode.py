"""GPU checks of msod_set_mode: the drop-in calls (full_convec_ijk,
full_diffusion_ijk through msod_convec_ijk / msod_diffusion_ijk, FP32
outputs) compute what the explicit entry points of each form compute."""
import numpy as np
import pytest

from minisod2d_gb300 import capi, kernels, learn, workload
from tests import refimpl

pytestmark = pytest.mark.gpu


@pytest.fixture
def mode():
    yield kernels.set_mode
    kernels.set_mode()


def _dev(cuda, P=5, nx=3, kind=1, seed=3, mu=1e-3):
    cfg = workload.Config("t", P, nx, 0.05, kind, 8, seed)
    host = workload.HostCase(cfg)
    rng = np.random.default_rng(seed)
    host.mu_e = (mu * rng.random(host.mu_e.size)).astype(np.float32)
    host.mu_sgs = (0.5 * mu * rng.random(host.mu_sgs.size)).astype(np.float32)
    return workload.DeviceCase(host, device=cuda)


def _close(a, b, tol):
    for x, y in zip(a, b):
        e = refimpl.rel_l2(x.double().cpu().numpy(), y.double().cpu().numpy())
        assert e < tol, e


def _p_from_T(dev):
    return dev.rho * float(learn.RGAS) * dev.Tem


def _plain_nu(dev, p):
    import torch

    mu = torch.empty(dev.nelem * dev.cfg.nnode, device=dev.rho.device)
    nu = torch.empty(dev.nelem, device=dev.rho.device)
    nm = torch.empty(dev.nelem, device=dev.rho.device)
    capi.call("msod_entropy_viscosity", *learn._geo(dev), learn._p(dev.rho), learn._p(dev.u), learn._p(p),
              float(learn.GAMMA), float(learn.CE), float(learn.CMAX), 1, learn._p(mu), learn._p(nu), learn._p(nm),
              torch.cuda.current_stream().cuda_stream)
    return nu


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_mode_precision(cuda, mode, prec):
    dev = _dev(cuda)
    ref_c = [x.float() for x in dev.convec_mixed(prec)]
    ref_d = [x.float() for x in dev.diffu_mixed(prec)]
    mode(prec)
    _close([x.clone() for x in dev.convec()], ref_c, 1e-6)
    _close([x.clone() for x in dev.diffu()], ref_d, 1e-6)
    mode()
    plain = [x.clone() for x in dev.convec()]
    _close(plain, ref_c, 1e-3)  # sanity: the plain kernels are near, not equal


def test_mode_plain_estimator(cuda, mode):
    dev = _dev(cuda)
    nu = _plain_nu(dev, _p_from_T(dev))
    ref = [x.clone() for x in learn.diffusion_ijk_nu(dev, nu)]
    mode("fp32", "plain")
    _close([x.clone() for x in dev.diffu()], ref, 1e-5)
    # with mixed precision too
    ref16 = [x.float() for x in dev.diffu_mixed("fp16", nu_elem=nu)]
    mode("fp16", "plain")
    _close([x.clone() for x in dev.diffu()], ref16, 1e-5)


def test_mode_learned(cuda, mode):
    import torch

    dev = _dev(cuda, P=4, nx=4)
    m = learn.Mlp(seed=2)
    w, norm = m.params()
    norm = norm.copy()
    norm[24:36] = -1e30  # no fallback: every element from the network
    norm[36:48] = 1e30
    m.set_params(None, norm)
    ref, nu_ref, _ = learn.diffusion_learned(m, dev, out=[torch.empty_like(x) for x in (dev.Dmass, dev.Dmom,
                                                                                        dev.Dener)], from_T=True)
    ref = [x.clone() for x in ref]
    mode("fp32", "learned", m)
    _close([x.clone() for x in dev.diffu()], ref, 1e-5)
    ref16 = [x.float() for x in dev.diffu_mixed("fp16", nu_elem=nu_ref)]
    mode("fp16", "learned", m)
    _close([x.clone() for x in dev.diffu()], ref16, 1e-5)
