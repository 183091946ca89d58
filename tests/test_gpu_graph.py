"""The drop-in calls inside a CUDA graph.

A host that repeats the same step can capture it once and replay it: the
calls issue only capturable stream work (memsets, device-to-device copies
into the constant bank, kernel launches) once their library buffers exist,
which the first eager call allocates."""
import numpy as np
import pytest

from minisod2d_gb300 import workload
from tests import refimpl

pytestmark = pytest.mark.gpu


def test_step_captured_in_a_cuda_graph(cuda):
    import torch

    dev = workload.DeviceCase(workload.HostCase(workload.Config("g", 4, 6, 0.05, 1, 8, 3)), device=cuda)
    rng = np.random.default_rng(0)
    dev.mu_e.copy_(torch.as_tensor((1e-3 * rng.random(dev.mu_e.numel())).astype(np.float32)))
    tet = workload.TetCase(dev.host, device=cuda)
    eager = [x.clone() for x in list(dev.convec()) + list(dev.diffu()) + list(tet.convec()) + list(tet.diffu())]
    torch.cuda.synchronize()
    outs = [dev.Rmass, dev.Rmom, dev.Rener, dev.Dmass, dev.Dmom, dev.Dener] + list(tet.R) + list(tet.D)
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(device=cuda)
    with torch.cuda.stream(side):
        for x in outs:
            x.fill_(1e9)
        with torch.cuda.graph(g, stream=side):
            dev.convec()
            dev.diffu()
            tet.convec()
            tet.diffu()
    for _ in range(3):
        for x in outs:
            x.fill_(-7.0)
        g.replay()
    torch.cuda.synchronize()
    for a, b in zip(outs, eager):
        assert refimpl.rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 1e-6


def test_one_call_step_captured_in_a_cuda_graph(cuda):
    """msod_convec_diffusion_ijk (one kernel at porder 4) replays from a graph to the eager results."""
    import torch

    dev = workload.DeviceCase(workload.HostCase(workload.Config("g", 4, 6, 0.05, 1, 8, 3)), device=cuda)
    rng = np.random.default_rng(1)
    dev.mu_e.copy_(torch.as_tensor((1e-3 * rng.random(dev.mu_e.numel())).astype(np.float32)))
    c, d = dev.convec_diffu()
    eager = [x.clone() for x in list(c) + list(d)]
    torch.cuda.synchronize()
    outs = [dev.Rmass, dev.Rmom, dev.Rener, dev.Dmass, dev.Dmom, dev.Dener]
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(device=cuda)
    with torch.cuda.stream(side):
        with torch.cuda.graph(g, stream=side):
            dev.convec_diffu()
    for _ in range(3):
        for x in outs:
            x.fill_(-7.0)
        g.replay()
    torch.cuda.synchronize()
    for a, b in zip(outs, eager):
        assert refimpl.rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 1e-6
