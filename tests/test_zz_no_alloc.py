"""pfc_segment_noalloc, the allocation-free segment entry point, against
pfc_segment.

Some callers cannot allocate device memory while they run the sieve: a server
that has reserved the whole GPU under its own budget and admits work against
it, or a host whose other streams must not be stalled by the synchronising
cudaMalloc/cudaFree.  For them the C ABI offers pfc_segment_noalloc, which works
in one static device array and writes only into buffers the caller passes.

Here the test plays that caller: it allocates the hit and totals buffers
itself (with torch), calls the entry point through the C ABI twice in a row on
different searches, and requires each result to equal what the allocating
entry point (pfc_segment) gives for the same segment.  The results are integers,
so the tolerance is zero: equal totals and equal sorted hit lists.  The file is
collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

pfc = pytest.importorskip("pfcsieve_gb300")
torch = pytest.importorskip("torch")

from oracle import oracle as o  # noqa: E402  (canonical hit order)

pytestmark = pytest.mark.gpu

# (mode, nmin, nmax, p_lo, p_hi): combined search on class-32 p, primorial on
# class-64 p, factorial with p <= n (Wilson hits)
CASES = [
    (5, 101, 20000, 10**9, 10**9 + 2 * 10**6),
    (2, 2000, 60000, 2**40, 2**40 + 3 * 10**6),
    (1, 101, 5000, 3, 50000),
]


def with_allocation(mode, nmin, nmax, lo, hi):
    with pfc.Context(0) as ctx, pfc.Job(ctx, mode, nmin, nmax, lo, hi) as job:
        job.segment(lo, hi)
        termsum, count = job.totals()
        hits = o.sort_factors(job.drain_hits())
    return termsum, count, hits


def without_allocation(mode, nmin, nmax, lo, hi, cap=1 << 16):
    hits = torch.zeros(cap * pfc.FACTOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    totals = torch.zeros(4, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = pfc.lib().pfc_segment_noalloc(mode, nmin, nmax, lo, hi, ctypes.c_void_p(hits.data_ptr()), cap,
                                       ctypes.c_void_p(totals.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, pfc.status_string(rc)
    t = totals.cpu().numpy().view(np.uint64)
    n = int(t[2])
    assert n <= cap
    h = hits[: n * pfc.FACTOR_DTYPE.itemsize].cpu().numpy().view(pfc.FACTOR_DTYPE)
    return int(t[0]), int(t[1]), o.sort_factors(h), int(t[3])


def test_two_calls_match_the_allocating_path():
    torch.cuda.init()
    for case in CASES[:2] + CASES[2:]:   # two calls in a row, then a third on the same array
        want = with_allocation(*case)
        termsum, count, hits, flags = without_allocation(*case)
        assert flags == 0
        assert (termsum, count) == want[:2], case
        assert np.array_equal(hits, want[2]), case


def test_repeated_call_clears_its_counters():
    case = CASES[0]
    first = without_allocation(*case)
    second = without_allocation(*case)
    assert first[:2] == second[:2] and np.array_equal(first[2], second[2])


def test_requests_beyond_the_limits_are_rejected():
    totals = torch.zeros(4, dtype=torch.int64, device="cuda")
    L = pfc.lib()
    # about 4e8 candidates: far more than 2^18
    rc = L.pfc_segment_noalloc(1, 101, 2000, 10**9, 2 * 10**10, None, 0,
                               ctypes.c_void_p(totals.data_ptr()), None)
    assert rc == -1
    # n range wider than 2^22
    rc = L.pfc_segment_noalloc(1, 101, 101 + (1 << 22) + 1, 10**9, 10**9 + 1000, None, 0,
                               ctypes.c_void_p(totals.data_ptr()), None)
    assert rc == -1
