"""Multi-rank host logic of bench.py on CPU: world_size 2 over gloo (127.0.0.1)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    r, local, w = bench.dist_setup()
    bench.barrier(w)
    m = bench.max_over_ranks(10.0 + r, w, torch.device("cpu"))
    bench.barrier(w)
    q.put((r, w, m))
    dist.destroy_process_group()


def test_two_rank_max_timing():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(o[0] for o in out) == [0, 1]
    assert all(o[1] == 2 and o[2] == 11.0 for o in out)  # max over ranks
