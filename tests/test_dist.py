"""Multi-rank logic on CPU (gloo, world size 2): bench.py's p-range shards for
weak scaling are contiguous, disjoint and equal, the reported time is the maximum
over ranks, and the shards of one search combine into the whole search (checksum
terms add, counts add, hits concatenate).  No data-path collective exists:
candidates are independent."""
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


def _shard_worker(rank, world, port, out):
    """Each rank sieves its half of a p range with the oracle; the halves'
    checksum terms add (mod 2^64), their candidate counts add and their hits
    concatenate, as the shards of a search combine."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as o
    mode, nmin, nmax, lo, hi = 5, 101, 3000, 10**6, 10**6 + 2 * 10**5
    cut = lo + (hi - lo) * rank // world, lo + (hi - lo) * (rank + 1) // world
    cands = o.candidates(*cut)
    hits, term, _ = o.sieve(mode, nmin, nmax, cands, threads=1)
    parts = [None] * world
    dist.all_gather_object(parts, (int(term), len(cands), hits.tolist()))
    if rank == 0:
        out.put(parts)
    dist.barrier()
    dist.destroy_process_group()


def test_shard_results_combine_to_the_whole_search():
    import numpy as np
    from oracle import oracle as o
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    mode, nmin, nmax, lo, hi = 5, 101, 3000, 10**6, 10**6 + 2 * 10**5
    cands = o.candidates(lo, hi)
    hits, term, _ = o.sieve(mode, nmin, nmax, cands, threads=1)
    assert sum(t for t, _, _ in parts) % 2**64 == int(term)
    assert sum(n for _, n, _ in parts) == len(cands)
    merged = [tuple(h) for _, _, hs in parts for h in hs]
    assert sorted(merged) == sorted(tuple(h) for h in hits.tolist())
