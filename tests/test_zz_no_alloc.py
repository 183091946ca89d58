"""The allocation-free table validation, through the C ABI (collected last).

msod_check_element_tables_noalloc serves callers that cannot let the library
cudaMalloc (an OpenACC-owned device pool, a capped allocator, allocations that
must precede CUDA-graph capture).  Its verdict must equal that of
msod_check_element_tables on the same inputs, call after call, and further calls
must not change the device's free memory.
"""
import ctypes as C
import os
import subprocess
import sys

import pytest

from minisod2d_gb300 import capi, workload

pytestmark = pytest.mark.gpu


def _args(dev, dlx, connec):
    P = dev.cfg.porder
    return [P, dev.nelem, dev.npoin, C.c_void_p(connec.data_ptr()), C.c_void_p(dlx.data_ptr()),
            C.c_void_p(dev.invAtoIJK.data_ptr()), C.c_void_p(dev.AtoI.data_ptr()), C.c_void_p(dev.AtoJ.data_ptr()),
            C.c_void_p(dev.AtoK.data_ptr()), None]


def test_noalloc_validation_matches_allocating_entry_point(cuda):
    import torch

    L = capi.lib()
    host = workload.HostCase(workload.Config("noalloc", 4, 2, 0.05, capi.MSOD_FIELDS_SMOOTH, 8, 0))
    dev = workload.DeviceCase(host, device=cuda)
    bad_dlx = dev.dlxigp_ip.clone()
    bad_dlx[7] += 1.0
    bad_con = dev.connec.clone()
    bad_con[3] = dev.npoin + 5
    cases = [("bad tables", _args(dev, bad_dlx, dev.connec)), ("good tables", _args(dev, dev.dlxigp_ip, dev.connec)),
             ("bad connec", _args(dev, dev.dlxigp_ip, bad_con)), ("good again", _args(dev, dev.dlxigp_ip, dev.connec))]
    torch.cuda.synchronize()
    codes = []
    for label, a in cases:  # consecutive calls: each must start from a cleared status word
        rc_ref = L.msod_check_element_tables(*a)
        msg_ref = L.msod_last_error_string()
        rc_new = L.msod_check_element_tables_noalloc(*a)
        msg_new = L.msod_last_error_string()
        assert rc_new == rc_ref, label
        assert msg_new == msg_ref, label
        codes.append(rc_new)
    assert codes == [capi.MSOD_ERR_BAD_TABLES, capi.MSOD_OK, capi.MSOD_ERR_BAD_TABLES, capi.MSOD_OK]
    # no allocation: the device's free memory is unchanged by further calls
    good = cases[1][1]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert L.msod_check_element_tables_noalloc(*good) == capi.MSOD_OK
    assert torch.cuda.mem_get_info()[0] == free0
    # sizes beyond the limits are rejected before any device work
    a = list(good)
    a[0] = capi.MSOD_MAX_PORDER + 1
    assert L.msod_check_element_tables_noalloc(*a) == capi.MSOD_ERR_PORDER
    a = list(good)
    a[1] = 1 << 30
    assert L.msod_check_element_tables_noalloc(*a) == capi.MSOD_ERR_INVALID_ARG
    assert b"int32" in L.msod_last_error_string()


FRESH = r"""
import ctypes as C, sys
sys.path.insert(0, %r)
from minisod2d_gb300 import capi, fem
L = capi.lib()   # loaded before the context exists: with CUDA_MODULE_LOADING=EAGER its module loads with it
import numpy as np, torch
dev = torch.device("cuda:0")
P = 4
t = fem.element_tables(P)
con, coord, nelem, npoin = fem.structured_mesh(P, 3, 3, 3, t, 0.0, 0)
d = {k: torch.from_numpy(np.ascontiguousarray(t[k])).to(dev)
     for k in ("dlxigp_ip", "invAtoIJK", "AtoI", "AtoJ", "AtoK", "dNgp", "wgp")}
connec = torch.from_numpy(con).to(dev)
args = [P, nelem, npoin] + [C.c_void_p(x.data_ptr()) for x in (connec, d["dlxigp_ip"], d["invAtoIJK"], d["AtoI"],
                                                               d["AtoJ"], d["AtoK"])] + [None]
# Before the measured window, one launch of another kernel of the library that allocates
# nothing (elem_jacobian into torch buffers): the driver sets up state of its own at the first
# launch from the library's module (8 MiB on this GPU), which belongs to no library call.
n = (P + 1) ** 3
d_coord = torch.from_numpy(coord).to(dev)
He = torch.empty(9 * nelem * n, device=dev)
gp = torch.empty(nelem * n, device=dev)
torch.cuda.synchronize()
free_w0 = torch.cuda.mem_get_info()[0]
assert L.msod_elem_jacobian(P, nelem, npoin, C.c_void_p(connec.data_ptr()), C.c_void_p(d_coord.data_ptr()),
                            C.c_void_p(d["dNgp"].data_ptr()), C.c_void_p(d["wgp"].data_ptr()),
                            C.c_void_p(gp.data_ptr()), C.c_void_p(He.data_ptr()), None) == 0
torch.cuda.synchronize()
print("WARMUP first launch from the library's module took %%d bytes" %% (free_w0 - torch.cuda.mem_get_info()[0]))
free0 = torch.cuda.mem_get_info()[0]
rcs = [L.msod_check_element_tables_noalloc(*args) for _ in range(5)]
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
rc_alloc = L.msod_check_element_tables(*args)   # the allocating entry point, as a control
torch.cuda.synchronize()
free2 = torch.cuda.mem_get_info()[0]
print("RESULT", rcs, free0, free1, rc_alloc, free2)
""" % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_noalloc_allocates_nothing_in_a_fresh_process(cuda):
    """In a fresh process (inputs built by torch, the library's module loaded eagerly with the
    context, one launch of another allocation-free library kernel beforehand), five calls of the
    allocation-free entry point -- the first with its per-device set-up included -- leave the
    device's free memory unchanged."""
    env = dict(os.environ, CUDA_MODULE_LOADING="EAGER")
    out = subprocess.run([sys.executable, "-c", FRESH], capture_output=True, text=True, env=env, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    print("\n".join(x for x in out.stdout.splitlines() if x.startswith("WARMUP")))
    line = [x for x in out.stdout.splitlines() if x.startswith("RESULT")][-1]
    rcs, rest = line[len("RESULT "):].split("]")
    assert [int(x) for x in rcs.strip(" [").split(",")] == [capi.MSOD_OK] * 5
    free0, free1, rc_alloc, free2 = (int(x) for x in rest.split())
    assert free1 == free0
    assert rc_alloc == capi.MSOD_OK
    # The control: the allocating entry point's first call takes device memory where the
    # measurement can see it (recorded, not required: the driver may sub-allocate).
    print("control: the allocating entry point changed free memory by %d bytes" % (free1 - free2))
