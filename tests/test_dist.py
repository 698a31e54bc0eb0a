"""Multi-rank logic of bench.py on CPU (gloo, world size 2): p-range shards
for weak scaling are contiguous, disjoint and equal, and the reported time is the
maximum over ranks.  No data-path collective exists: candidates are independent."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    wl = bench.WORKLOADS["combined"]
    lo, hi = bench.shard(wl, rank)
    shards = [None] * world
    dist.all_gather_object(shards, (lo, hi))
    t = bench.barrier_max(dist, 1.5 + rank)
    if rank == 0:
        out.put((shards, t))
    dist.barrier()
    dist.destroy_process_group()


def test_weak_scaling_shards_and_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    shards, t = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (a0, b0), (a1, b1) = shards
    assert b0 == a1 and (b0 - a0) == (b1 - a1) == 10**8
    assert t == 2.5
