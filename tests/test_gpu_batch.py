"""The batch engine (pfc_batch_*) against the per-job path and the oracle.

Every search run inside a batch must give exactly what it gives alone
(pfc_job_run): the same wrapping checksum-term sum, candidate count and raw hit
multiset, whatever else shares the GPU with it and whenever it joined.  Small
cases are also checked against the oracle directly.
"""
import os

import numpy as np
import pytest

from oracle import oracle as o

pfc = pytest.importorskip("pfcsieve_gb300")

pytestmark = pytest.mark.gpu

THREADS = min(os.cpu_count() or 1, 64)

# every mode, both size classes, p <= n (Wilson hits), tiny n ranges, a primorial
# range with no prime n, and nmin == nmax
MIX = [
    (5, 101, 20000, 10**9, 10**9 + 2 * 10**6),
    (1, 101, 5000, 3, 50000),
    (2, 2000, 60000, 2**40, 2**40 + 3 * 10**6),
    (4, 150, 30000, 2**31 - 10**6, 2**31 + 10**6),
    (2, 101, 40000, 1000, 3 * 10**6),
    (1, 30000, 31000, 2**33, 2**33 + 5 * 10**6),
    (5, 5000, 9000, 10**5, 4 * 10**6),
    (4, 101, 102, 10**6, 2 * 10**6),
    (2, 114, 126, 10**7, 10**7 + 10**6),
    (1, 500, 500, 10**6, 10**6 + 10**5),
    # class-64 regimes: below, across and above 2^64/3, across 2^63
    (5, 2000, 6000, 0x5555555555555556 - 200000, 0x5555555555555556),
    (2, 2000, 30000, 0x5555555555555556 - 100000, 0x5555555555555556 + 100000),
    (4, 2000, 6000, 2**63 - 100000, 2**63 + 100000),
    (1, 2000, 6000, 2**64 - 200000, 2**64 - 1),
]


def alone(ctx, case):
    with pfc.Job(ctx, *case) as job:
        hits = job.run()
        termsum, count = job.totals()
    return termsum, count, o.sort_factors(hits)


def batched(b, jid):
    st = b.status(jid)
    assert st.done == 1 and st.status == 0, (jid, st.status)
    return st.term_checksum, st.primecount, o.sort_factors(b.hits(jid))


@pytest.fixture(scope="module")
def ctx():
    with pfc.Context(0) as c:
        yield c


def test_batch_equals_jobs_alone(ctx):
    with pfc.Batch(ctx) as b:
        ids = [b.submit(*c) for c in MIX]
        b.run()
        for case, jid in zip(MIX, ids):
            got = batched(b, jid)
            want = alone(ctx, case)
            assert got[:2] == want[:2], case
            assert np.array_equal(got[2], want[2]), case


def test_batch_matches_oracle_on_small_cases(ctx):
    cases = [MIX[1], MIX[4], MIX[6]]
    with pfc.Batch(ctx) as b:
        ids = [b.submit(*c) for c in cases]
        b.run()
        for case, jid in zip(cases, ids):
            termsum, count, hits = batched(b, jid)
            mode, nmin, nmax, pmin, pmax = case
            cands = o.candidates(pmin, pmax)
            ohits, oterm, _ = o.sieve(mode, nmin, nmax, cands, threads=THREADS)
            assert count == len(cands), case
            assert termsum == oterm, case
            assert np.array_equal(hits, ohits), case


# class 64 below 2^64/3: the batch sets these searches up on the tensor cores
# at admission (one launch per search) and walks them in its windows
TC_MIX = [MIX[2], MIX[5], MIX[10], MIX[11],
          (5, 30000, 33000, 2**45, 2**45 + 2 * 10**6),
          (4, 101, 50000, 2**55, 2**55 + 10**6),
          (2, 60000, 60300, 2**50, 2**50 + 10**6),   # a primorial n range without primes: setup windows
          # programs above the tensor-core thresholds (kernels.cuh): class 64,
          # class 32, and both classes in one search
          (1, 400000, 400100, 2**45, 2**45 + 2 * 10**6),
          (5, 300000, 300100, 2**50, 2**50 + 10**6),
          (1, 300000, 300200, 10**9, 10**9 + 10**6),
          (5, 300000, 300100, 2**31 - 10**6, 2**31 - 10),
          (4, 600000, 600100, 2**31 - 10**5, 2**31 + 10**5)]


def test_batch_tensor_core_setup_equals_the_integer_setup(ctx):
    """Searches of class 32 and of the lazy class-64 range in a batch whose
    context sets them up on the tensor cores give exactly what they give
    alone with the
    integer-pipe setup."""
    with pfc.Context(0) as ref:
        ref.set_setup_tc(False)
        want = [alone(ref, case) for case in TC_MIX]
    with pfc.Batch(ctx) as b:
        ids = [b.submit(*c) for c in TC_MIX]
        b.run()
        for case, jid, w in zip(TC_MIX, ids, want):
            got = batched(b, jid)
            assert got[:2] == w[:2], case
            assert np.array_equal(got[2], w[2]), case


def test_batch_tensor_core_setup_matches_the_oracle(ctx):
    # programs above the tensor-core thresholds (kTcMinWords64 = 480, kTcMinWords32 = 448 words)
    cases = [(1, 400000, 400400, 2**40, 2**40 + 3 * 10**4), (5, 300000, 300300, 2**47, 2**47 + 3 * 10**4),
             (2, 600000, 600600, 2**61, 2**61 + 3 * 10**4), (1, 300000, 300400, 10**8, 10**8 + 3 * 10**4)]
    with pfc.Batch(ctx) as b:
        ids = [b.submit(*c) for c in cases]
        b.run()
        for case, jid in zip(cases, ids):
            termsum, count, hits = batched(b, jid)
            mode, nmin, nmax, pmin, pmax = case
            cands = o.candidates(pmin, pmax)
            ohits, oterm, _ = o.sieve(mode, nmin, nmax, cands, threads=THREADS)
            assert count == len(cands), case
            assert termsum == oterm, case
            assert np.array_equal(hits, ohits), case


def test_jobs_joining_a_running_batch(ctx):
    """Continuous batching: searches submitted between iterations start at
    the next one and still give their stand-alone results."""
    first, later = MIX[:4], MIX[4:]
    with pfc.Batch(ctx, iteration_work=2e8) as b:
        ids = [b.submit(*c) for c in first]
        b.step()
        active, queued = b.step()
        assert active == len(first) and queued == 0   # still running when the others arrive
        ids += [b.submit(*c) for c in later]
        active, queued = b.step()
        assert queued == 0 and active >= 1
        assert not b.status(ids[0]).done                # overlapped with the newcomers
        b.run()
        assert b.iterations >= 4
        for case, jid in zip(first + later, ids):
            got = batched(b, jid)
            want = alone(ctx, case)
            assert got[:2] == want[:2], case
            assert np.array_equal(got[2], want[2]), case


def test_finished_search_is_released(ctx):
    with pfc.Batch(ctx) as b:
        jid = b.submit(*MIX[1])
        b.run()
        b.release(jid)
        with pytest.raises(pfc.PFCError):
            b.status(jid)


def test_invalid_searches_are_rejected(ctx):
    with pfc.Batch(ctx) as b:
        for bad in [(3, 101, 200, 10**6, 2 * 10**6), (1, 100, 200, 10**6, 2 * 10**6),
                    (1, 101, 200, 2, 10**6), (1, 101, 200, 10**6, 10**6),
                    (1, 101, 200, 2**40, 2**40 + 10**13)]:     # ~3.6e11 candidates: too many to hold
            with pytest.raises(pfc.PFCError):
                b.submit(*bad)


def test_latency_policy_gives_the_same_results(ctx):
    """Shortest-remaining-work-first windows change only the order of work:
    searches submitted between iterations under the latency policy still
    equal their stand-alone results, and the small ones finish first."""
    with pfc.Batch(ctx, iteration_work=5e8, policy=pfc.BATCH_LATENCY) as b:
        ids = []
        for k, case in enumerate(MIX):
            ids.append(b.submit(*case))
            if k % 3 == 2:
                b.step()
        finished = []
        while True:
            active, queued = b.step()
            for jid in ids:
                if jid not in finished and b.status(jid).done:
                    finished.append(jid)
            if active == 0 and queued == 0:
                break
        for case, jid in zip(MIX, ids):
            got = batched(b, jid)
            want = alone(ctx, case)
            assert got[:2] == want[:2], case
            assert np.array_equal(got[2], want[2]), case
        # the largest search of the mix (by candidates x n) is not among the first to finish
        big = max(range(len(MIX)), key=lambda i: (MIX[i][4] - MIX[i][3]) * (MIX[i][2] - MIX[i][1]))
        assert finished.index(ids[big]) >= len(MIX) // 2


def test_hit_overflow_reruns_the_searches_alone(ctx):
    """A hit list too small for an iteration's hits: the searches of that
    iteration are redone alone, and every result still equals the stand-alone
    one.  (p <= n makes every candidate hit: Wilson's theorem.)"""
    cases = [MIX[1], (5, 101, 6000, 3, 6000), MIX[3]]
    with pfc.Batch(ctx) as b:
        b.set_hit_capacity(64)
        ids = [b.submit(*c) for c in cases]
        b.run()
        for case, jid in zip(cases, ids):
            got = batched(b, jid)
            want = alone(ctx, case)
            assert got[:2] == want[:2], case
            assert np.array_equal(got[2], want[2]), case
        assert len(got[2]) > 64 or len(batched(b, ids[1])[2]) > 64


def test_hit_capacity_is_fixed_while_searches_run(ctx):
    with pfc.Batch(ctx, iteration_work=1e8) as b:
        b.submit(*MIX[0])
        b.step()
        with pytest.raises(pfc.PFCError):
            b.set_hit_capacity(128)
        b.run()


def test_memory_budget_admission():
    """A context whose budget holds only some of the searches at once: the
    rest wait in the queue until running ones retire, and every result still
    equals the stand-alone one."""
    cases = [(1, 2000, 6000, 2**40 + k * 10**8, 2**40 + k * 10**8 + 2 * 10**7) for k in range(6)]
    with pfc.Context(0, budget=96 << 20) as small:
        # iterations short enough that the admitted searches are still
        # running while the others wait for their memory
        with pfc.Batch(small, iteration_work=5e8) as b:
            ids = [b.submit(*c) for c in cases]
            max_active, saw_queue = 0, False
            while True:
                active, queued = b.step()
                max_active = max(max_active, active)
                saw_queue |= active > 0 and queued > 0
                if active == 0 and queued == 0:
                    break
            assert saw_queue and max_active < len(cases)
            got = [batched(b, jid) for jid in ids]
    with pfc.Context(0) as big:
        for case, g in zip(cases, got):
            want = alone(big, case)
            assert g[:2] == want[:2], case
            assert np.array_equal(g[2], want[2]), case
