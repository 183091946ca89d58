"""Kernel calls of different porders issued on two streams without
synchronisation between them: each call has its own element-table area and
constant-bank matrices, so the results equal the sequential ones (up to the
order of the atomic node sums)."""
import pytest

from minisod2d_gb300 import workload
from tests import refimpl

pytestmark = pytest.mark.gpu


def test_interleaved_porders_on_two_streams(cuda):
    import torch

    a = workload.DeviceCase(workload.HostCase(workload.Config("a", 4, 6, 0.05, 1, 8, 1)), device=cuda)
    b = workload.DeviceCase(workload.HostCase(workload.Config("b", 2, 9, 0.05, 0, 8, 2)), device=cuda)
    ref = {}
    for name, dev in (("a", a), ("b", b)):
        ref[name] = [x.clone() for x in list(dev.convec()) + list(dev.diffu())]
    torch.cuda.synchronize()
    sa, sb = torch.cuda.Stream(device=cuda), torch.cuda.Stream(device=cuda)
    for _ in range(3):
        for dev, s in ((a, sa), (b, sb), (a, sa), (b, sb)):
            dev.convec(stream=s.cuda_stream)
            dev.diffu(stream=s.cuda_stream)
    torch.cuda.synchronize()
    for name, dev in (("a", a), ("b", b)):
        got = [dev.Rmass, dev.Rmom, dev.Rener, dev.Dmass, dev.Dmom, dev.Dener]
        for g, r in zip(got, ref[name]):
            assert refimpl.rel_l2(g.cpu().numpy(), r.cpu().numpy()) < 1e-6, name
