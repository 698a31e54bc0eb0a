"""Host logic of the mixed workload and the request loop (no GPU needed).

* mixed_jobs draws the mixed workload deterministically from its seed and
  keeps every search inside the ranges the C ABI accepts;
* poisson_arrivals is a seeded Poisson process at the requested rate;
* fcfs_latencies is the latency of a single first-come-first-served server,
  checked against a direct event simulation.
"""
import math
import os

import numpy as np
import pytest

serving = pytest.importorskip("pfcsieve_gb300.serving")


def test_mixed_jobs_are_deterministic_and_in_range():
    a = serving.mixed_jobs(512, seed=0)
    b = serving.mixed_jobs(512, seed=0)
    assert a == b
    assert serving.mixed_jobs(512, seed=1) != a
    assert len(a) == 512
    for s in a:
        assert s.mode in (1, 2, 4)
        assert 101 <= s.nmin < 10**7
        assert 10**3 <= s.nmax - s.nmin <= 10**6
        assert s.nmax < 2**31
        assert 10**5 <= s.pmax - s.pmin <= 10**8
        assert 10**8 <= s.pmin <= 2**63
        assert s.pmax < 2**64


def test_mixed_jobs_distribution():
    jobs = serving.mixed_jobs(4096, seed=3)
    modes = np.bincount([s.mode for s in jobs], minlength=5)
    for m in (1, 2, 4):
        assert abs(modes[m] / len(jobs) - 1 / 3) < 0.04
    # log-uniform lengths: the median is near the geometric mean of the bounds
    nl = np.median([math.log10(s.nmax - s.nmin) for s in jobs])
    pl = np.median([math.log10(s.pmax - s.pmin) for s in jobs])
    assert abs(nl - 4.5) < 0.15 and abs(pl - 6.5) < 0.15


def test_first_searches_of_a_seed_are_a_prefix():
    """The benchmark's sample is the first k searches of the 512-search set."""
    assert serving.mixed_jobs(512, seed=0)[:32] == serving.mixed_jobs(32, seed=0)


def test_poisson_arrivals():
    t = serving.poisson_arrivals(20000, 200.0, seed=1)
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 200.0) < 2e-4
    assert abs(gaps.std() - 1 / 200.0) < 3e-4          # exponential: std == mean
    assert np.array_equal(t, serving.poisson_arrivals(20000, 200.0, seed=1))


def test_fcfs_latencies_match_an_event_simulation():
    rng = np.random.default_rng(5)
    arr = np.cumsum(rng.exponential(0.1, 300))
    svc = rng.exponential(0.12, 300)
    lat = serving.fcfs_latencies(arr, svc)
    clock = 0.0
    for i in range(300):
        start = max(clock, arr[i])
        clock = start + svc[i]
        assert abs(lat[i] - (clock - arr[i])) < 1e-9
    # an idle server: latency is the service time
    assert np.allclose(serving.fcfs_latencies([0.0, 10.0], [1.0, 2.0]), [1.0, 2.0])


def test_batched_roofline_counts():
    """bench.mixed_roofline: per search, candidates x (setup words x word cost
    + squarings x squaring cost + algorithmic walk steps x step cost); with
    the tensor-core setup on, programs below its thresholds keep the
    integer-pipe word cost."""
    import types
    pfc = pytest.importorskip("pfcsieve_gb300")
    import bench
    peaks = {"imad": 20e12, "mul_hi": 8e12, "imad_wide": 10e12, "iadd_xor": 40e12}
    w, h = 2.0, 2.5
    S = serving.Search
    jobs = [S(1, 300000, 301000, 10**9, 10**9 + 10**6),      # class 32, n!: 1000 steps, 687 words
            S(5, 200000, 201000, 2**40, 2**40 + 10**6),      # class 64 below 2^64/3, n! and composite n: 600 words
            S(2, 5000, 6000, 2**63 + 10**6, 2**63 + 2 * 10**6),  # class 64 above 2^64/3, prime n only
            S(1, 5000, 6000, 10**9, 10**9 + 10**6),          # class 32, 21 words
            S(4, 5000, 6000, 2**40, 2**40 + 10**6)]          # class 64 below 2^64/3, composite n only: 17 words
    out = {i: types.SimpleNamespace(primecount=100 + i) for i in range(len(jobs))}

    def nprimes(a, b):
        return sum(1 for q in range(a, b) if all(q % d for d in range(2, int(q ** 0.5) + 1)))
    p3, p2, p5 = nprimes(300000, 301000), nprimes(200000, 201000), nprimes(5000, 6000)
    w1, s1 = pfc.setup_program_size(1, 300000)
    w5, s5 = pfc.setup_program_size(5, 200000)
    w2, s2 = pfc.setup_program_size(2, 5000, wide=False)
    v1, t1 = pfc.setup_program_size(1, 5000)
    v4, t4 = pfc.setup_program_size(4, 5000)
    assert w1 >= bench.TC_MIN_WORDS[32] and w5 >= bench.TC_MIN_WORDS[64]
    assert v1 < bench.TC_MIN_WORDS[32] and v4 < bench.TC_MIN_WORDS[64]
    for setup_tc, word32, word64 in ((False, 36 * w + 2, 76 * w + 3), (True, 1.5 * w + 1, 5 * w + 1.5)):
        # with the tensor-core setup the words' fold leaves the integer pipe
        # (half a reduction and half a product per 896-bit word remain)
        tc_s = 0.5 if setup_tc else 0.0
        r = bench.mixed_roofline(jobs, out, 2.0, peaks, tc_s=tc_s, setup_tc=setup_tc)
        want = (100 * (w1 * word32 + s1 * (w + 1 + h) + 1000 * (2 * w + 1))
                + 101 * (w5 * word64 + s5 * (8 * w + 2) + (2000 - p2) * (4 * w + 1))
                + 102 * (w2 * (8 * w + 2) + s2 * (8 * w + 2) + p5 * (7 * w + 2))
                + 103 * (v1 * (36 * w + 2) + t1 * (w + 1 + h) + 1000 * (2 * w + 1))
                + 104 * (v4 * (76 * w + 3) + t4 * (8 * w + 2) + (1000 - p5) * (4 * w + 1)))
        assert abs(r["alg_ops"] - want) < 1e-6 * want
        assert abs(r["frac"] - want / 2.0 / 20e12) < 1e-9
        if setup_tc:
            flops = 2 * (100 * w1 * 112 * 4 + 101 * w5 * 112 * 8)
            assert r["tensor_setup"]["flops"] == flops
            assert abs(r["tensor_setup"]["achieved_tflops"] - flops / 2.0 / 1e12) < 1e-12
        else:
            assert r["tensor_setup"] is None
    assert p3 > 0


def test_roofline_thresholds_follow_the_kernels():
    """bench.TC_MIN_WORDS restates kTcMinWords32/kTcMinWords64 of kernels.cuh."""
    import re
    import bench
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "pfcsieve_gb300", "csrc", "kernels.cuh")).read()
    got = {int(c): int(v) for c, v in re.findall(r"constexpr uint64_t kTcMinWords(32|64) = (\d+);", src)}
    assert got == bench.TC_MIN_WORDS
