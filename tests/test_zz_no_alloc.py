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

# one call whose p range holds both size classes (it crosses 2^31), the
# combined search on class-64 p below 2^64/3 (lazy steps, 896-bit setup
# words), and segments at or above 2^64/3 (canonical 64-bit steps)
MORE_CASES = [
    (5, 101, 5000, 2**31 - 10**6, 2**31 + 10**6),
    (5, 1000, 8000, 2**50, 2**50 + 10**6),
    (1, 101, 3000, 2**64 - 2 * 10**6, 2**64 - 1),
    (4, 500, 4000, 2**64 // 3 - 5 * 10**5, 2**64 // 3 + 5 * 10**5),
]


def with_allocation(mode, nmin, nmax, lo, hi):
    with pfc.Context(0) as ctx, pfc.Job(ctx, mode, nmin, nmax, lo, hi) as job:
        job.segment(lo, hi)
        termsum, count = job.totals()
        hits = o.sort_factors(job.drain_hits())
    return termsum, count, hits


def call(case, hits, cap, totals, stream=None):
    """One call through the C ABI into caller-owned device buffers."""
    mode, nmin, nmax, lo, hi = case
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    return pfc.lib().pfc_segment_noalloc(mode, nmin, nmax, lo, hi, ctypes.c_void_p(hits.data_ptr()), cap,
                                         ctypes.c_void_p(totals.data_ptr()), ctypes.c_void_p(stream))


def without_allocation(mode, nmin, nmax, lo, hi, cap=1 << 16):
    hits = torch.zeros(cap * pfc.FACTOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    totals = torch.zeros(4, dtype=torch.int64, device="cuda")
    rc = call((mode, nmin, nmax, lo, hi), hits, cap, totals)
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


@pytest.mark.parametrize("case", MORE_CASES)
def test_both_classes_and_the_canonical_class_64(case):
    want = with_allocation(*case)
    termsum, count, hits, flags = without_allocation(*case)
    assert flags == 0
    assert (termsum, count) == want[:2], case
    assert np.array_equal(hits, want[2]), case


def test_call_leaves_device_memory_unchanged():
    """After a first call on the device (which resolves the array's address),
    a call changes nothing in the device's free memory."""
    case = CASES[0]
    cap = 1 << 12
    hits = torch.zeros(cap * pfc.FACTOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    totals = torch.zeros(4, dtype=torch.int64, device="cuda")
    assert call(case, hits, cap, totals) == 0
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    assert call(case, hits, cap, totals) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_hits_beyond_the_capacity_are_counted_not_written():
    case = CASES[2]                      # factorial with p <= n: many hits
    full = with_allocation(*case)[2]
    slots = 16
    hits = torch.full((slots * pfc.FACTOR_DTYPE.itemsize,), 0xFF, dtype=torch.uint8, device="cuda")
    totals = torch.zeros(4, dtype=torch.int64, device="cuda")
    assert call(case, hits, 1, totals) == 0
    t = totals.cpu().numpy().view(np.uint64)
    assert int(t[2]) == len(full) > 1
    rec = hits.cpu().numpy().view(pfc.FACTOR_DTYPE)
    assert (full == rec[0]).any()
    assert (hits.cpu().numpy()[pfc.FACTOR_DTYPE.itemsize:] == 0xFF).all()


def test_candidate_overflow_sets_the_flag(monkeypatch):
    """More candidates than the call holds: flag bit 0, the true count, and no
    write beyond the capacity (the test lowers the capacity to 1000 through
    the library's environment setting; the p range holds about 4,800)."""
    case = (1, 101, 2000, 10**9, 10**9 + 10**5)
    want_count = with_allocation(*case)[1]
    monkeypatch.setenv("PFCSIEVE_NOALLOC_CAND_CAP", "1000")
    termsum, count, hits, flags = without_allocation(*case)
    assert flags & 1
    assert count == want_count > 1000
    monkeypatch.delenv("PFCSIEVE_NOALLOC_CAND_CAP")
    termsum, count, hits, flags = without_allocation(*case)
    assert flags == 0 and count == want_count


def test_call_on_a_capturing_stream_is_refused():
    """The call waits for its stream and copies from short-lived host memory,
    so on a stream under capture it returns PFC_ERR_STATE and enqueues
    nothing: the caller's capture stays valid."""
    cap = 1 << 10
    hits = torch.zeros(cap * pfc.FACTOR_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    totals = torch.zeros(4, dtype=torch.int64, device="cuda")
    x = torch.zeros(1, device="cuda")
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=side):
        x += 1
        rc = call(CASES[0], hits, cap, totals, stream=side.cuda_stream)
    assert rc == -7
    graph.replay()
    torch.cuda.synchronize()
    assert float(x.item()) == 1.0
