"""Multi-GPU is replicas only (independent chains / proposals, no collective on the data
path); the only exchange is the max-over-ranks timing bench.py reports.  Covered here
with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(10.0 * (rank + 1))
    rate = bench.whole_job_rate(world, 64, 5, ms)
    out.put((rank, ms, rate))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate in res:
        assert ms == 20.0                       # slowest rank bounds the job
        assert rate == pytest.approx(2 * 64 * 5 / 0.020)


def test_single_process_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
