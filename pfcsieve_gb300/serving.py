"""Mixed search workloads and the request loop over the batch engine.

The reference runs one search per process (main.cpp:219-323): a user with many
searches queues processes.  Here a queue of searches is served by one
pfc_batch on one GPU:

* mixed_jobs() draws a seeded mix of searches of uneven size: modes uniform
  over {n!, n#, n!/n#}, n-range length log-uniform in [1e3, 1e6] from n0
  uniform in [101, 1e7), p-range length log-uniform in [1e5, 1e8] from p0
  log-uniform in [1e8, 2^63].
* run_batched() runs a list of searches as one batch; run_plain() runs them
  one after the other, one search per launch sequence (pfc_job_run), as the
  reference would.
* serve() is the request loop: searches arrive by a Poisson process, join the
  running batch at the next iteration (continuous batching: the engine admits
  them as memory and slots free up), and each one's latency from arrival to
  result is recorded.
"""
import math
import time
from dataclasses import dataclass

import numpy as np

from . import BATCH_LATENCY, COMPOSITORIAL, FACTORIAL, PRIMORIAL, Batch, Job, PFCError

MODES = (FACTORIAL, PRIMORIAL, COMPOSITORIAL)


@dataclass(frozen=True)
class Search:
    mode: int
    nmin: int
    nmax: int
    pmin: int
    pmax: int

    def astuple(self):
        return (self.mode, self.nmin, self.nmax, self.pmin, self.pmax)


def mixed_jobs(count=512, seed=0, n_len=(1e3, 1e6), n0=(101, 10**7), p_len=(1e5, 1e8),
               p0=(1e8, 2.0**63)):
    """`count` searches drawn as described in the module docstring."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        mode = int(MODES[rng.integers(0, 3)])
        nl = int(math.exp(rng.uniform(math.log(n_len[0]), math.log(n_len[1]))))
        nmin = int(rng.integers(n0[0], n0[1]))
        pl = int(math.exp(rng.uniform(math.log(p_len[0]), math.log(p_len[1]))))
        pmin = int(math.exp(rng.uniform(math.log(p0[0]), math.log(p0[1]))))
        pmin = min(max(pmin, 3), 2**63)
        out.append(Search(mode, nmin, nmin + nl, pmin, pmin + pl))
    return out


def pairs_of(s, counts):
    """(p, n) pairs a search tests: candidates x n-range length."""
    return counts * (s.nmax - s.nmin)


@dataclass
class Outcome:
    term_checksum: int
    primecount: int
    hits: np.ndarray


def run_batched(ctx, searches, iteration_work=None, keep_hits=True):
    """All searches in one batch; returns ({index: Outcome}, seconds, timing dict)."""
    with Batch(ctx, iteration_work) as b:
        t0 = time.perf_counter()
        ids = [b.submit(*s.astuple()) for s in searches]
        b.run()
        dt = time.perf_counter() - t0
        out = {}
        for i, jid in enumerate(ids):
            st = b.status(jid)
            if st.status != 0:
                raise PFCError(st.status, "batched search %d" % i)
            out[i] = Outcome(st.term_checksum, st.primecount, b.hits(jid) if keep_hits else None)
            b.release(jid)
        return out, dt, b.timing()


def run_plain(ctx, searches, keep_hits=True):
    """One search after the other through pfc_job_run.

    Returns ({index: Outcome}, seconds, per-search service times, seconds
    spent building host tables in pfc_job_create)."""
    out = {}
    service = np.zeros(len(searches))
    create = 0.0
    t0 = time.perf_counter()
    for i, s in enumerate(searches):
        t1 = time.perf_counter()
        with Job(ctx, *s.astuple()) as job:
            create += time.perf_counter() - t1
            hits = job.run()
            termsum, count = job.totals()
        service[i] = time.perf_counter() - t1
        out[i] = Outcome(termsum, count, hits if keep_hits else None)
    return out, time.perf_counter() - t0, service, create


def fcfs_latencies(arrivals, service):
    """Latencies of a single first-come-first-served server with the given
    arrival and service times (the plain path serves one search at a time)."""
    lat = np.zeros(len(arrivals))
    free = 0.0
    for i, (a, s) in enumerate(zip(arrivals, service)):
        free = max(free, a) + s
        lat[i] = free - a
    return lat


def poisson_arrivals(count, rate, seed=1):
    """Arrival times (s from start) of `count` requests at mean `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=count))


def serve(ctx, searches, arrivals, iteration_work=5e10, keep_hits=False):
    """Request loop: submit each search when its arrival time has passed, step
    the batch while anything is queued or running, and collect results.  The
    batch runs the latency policy (shortest remaining work first) with short
    iterations.

    Returns (outcomes, latencies in s, makespan in s)."""
    with Batch(ctx, iteration_work, policy=BATCH_LATENCY) as b:
        t0 = time.perf_counter()
        pending = list(range(len(searches)))
        running = {}
        lat = np.zeros(len(searches))
        out = {}
        while pending or running:
            now = time.perf_counter() - t0
            while pending and arrivals[pending[0]] <= now:
                i = pending.pop(0)
                running[b.submit(*searches[i].astuple())] = i
            if not running:
                time.sleep(max(0.0, min(arrivals[pending[0]] - now, 0.01)))
                continue
            b.step()
            now = time.perf_counter() - t0
            for jid in list(running):
                st = b.status(jid)
                if st.done:
                    i = running.pop(jid)
                    if st.status != 0:
                        raise PFCError(st.status, "served search %d" % i)
                    lat[i] = now - arrivals[i]
                    out[i] = Outcome(st.term_checksum, st.primecount, b.hits(jid) if keep_hits else None)
                    b.release(jid)
        return out, lat, time.perf_counter() - t0
