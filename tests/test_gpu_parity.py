"""Parity of the CUDA path (through the C ABI) with the oracle and with the
reference's own golden vectors.  All tests need a GB300 (marker gpu).

Bar: bit-exact.  Candidates are compared as sorted lists, residues candidate
by candidate in the reference's representation (Montgomery, R = 2^64), hits
as sorted (p, |n|, type, nc) lists, and whole searches by the reference's
self-test triple (factorcount, primecount, checksum).
"""
import os

import numpy as np
import pytest

from oracle import oracle as o
from tests import goldens

pfc = pytest.importorskip("pfcsieve_gb300")

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx():
    c = pfc.Context(0)
    yield c
    c.close()


def run_segment(ctx, mode, nmin, nmax, pmin, pmax, lo=None, hi=None):
    lo = pmin if lo is None else lo
    hi = pmax if hi is None else hi
    with pfc.Job(ctx, mode, nmin, nmax, pmin, pmax) as job:
        job.segment(lo, hi)
        p, s0, s1 = job.segment_state()
        hits = o.sort_factors(job.drain_hits())
        termsum, count = job.totals()
    order = np.argsort(p, kind="stable")
    return p[order], s0[order], s1[order], hits, termsum, count


def oracle_terms(mode, s4s6s7):
    return goldens.terms_from_records(mode, s4s6s7)


# ------------------------------------------------------------ candidates

@pytest.mark.parametrize("lo,hi", [
    (3, 200000), (101, 5000), (113, 130), (42000, 90000),
    (10**9, 10**9 + 3 * 10**6), (2**32 - 200000, 2**32 + 200000),
    (2**62, 2**62 + 300000), (2**64 - 300000, 2**64 - 1), (4294967290, 4294967300),
])
def test_candidates_match_oracle(ctx, lo, hi):
    with pfc.Job(ctx, 1, 101, 102, lo, hi) as job:
        job.gen(lo, hi)
        job.setup()
        job.iterate(101, 102)
        job.check()
        p, _, _ = job.segment_state()
        _, count = job.totals()
    assert count == len(p)
    assert np.array_equal(np.sort(p), o.candidates(lo, hi))


# --------------------------------------------- reference kernel fixtures

def test_reference_fixture_segments(ctx):
    segs, _, _ = goldens.ref_segments()
    for s in segs:
        p, s0, s1, hits, termsum, count = run_segment(ctx, s["mode"], s["nmin"], s["nmax"],
                                                      s["pmin"], s["pmax"])
        assert np.array_equal(p, s["cands"]), s["mode"]
        ref = s["s4s6s7"]
        assert np.array_equal(s0, ref[:, 1]), (s["mode"], s["pmin"])
        if s["mode"] == 5:
            assert np.array_equal(s1, ref[:, 0]), (s["mode"], s["pmin"])
        assert np.array_equal(hits, s["hits"]), (s["mode"], s["pmin"])
        with np.errstate(over="ignore"):
            want = int(np.sum(oracle_terms(s["mode"], ref), dtype=np.uint64))
        assert termsum == want
        assert count == len(s["cands"])


# ------------------------------------------- oracle at random small sizes

@pytest.mark.parametrize("seed", range(6))
def test_random_segments_vs_oracle(ctx, seed):
    rng = np.random.default_rng(seed)
    mode = [1, 2, 4, 5][seed % 4]
    nmin = int(rng.integers(101, 30000))
    nmax = nmin + int(rng.integers(1, 5000))
    bits = int(rng.choice([20, 31, 33, 45, 63, 64]))
    pmin = int(rng.integers(3, 2**bits - 100000)) if bits < 64 else 2**64 - 2000000
    pmax = pmin + int(rng.integers(1000, 60000))
    p, s0, s1, hits, termsum, _ = run_segment(ctx, mode, nmin, nmax, pmin, pmax)
    cands = o.candidates(pmin, pmax)
    assert np.array_equal(p, cands)
    ohits, osum, terms = o.sieve(mode, nmin, nmax, cands, THREADS, want_terms=True)
    assert np.array_equal(s0, terms[:, 0])
    if mode == 5:
        assert np.array_equal(s1, terms[:, 2])
    assert np.array_equal(hits, ohits)
    assert termsum == osum


# class-64 arithmetic regimes: 128-bit setup words and lazy walk below
# 2^64/3, 64-bit setup words with the lazy walk up to 2^63, canonical above
LAZY_END = 0x5555555555555556


@pytest.mark.parametrize("lo", [LAZY_END - 120000, LAZY_END - 60000, 2**63 - 60000, 2**63 - 120000,
                                2**64 - 200000, 2**33])
@pytest.mark.parametrize("mode", [1, 2, 4, 5])
def test_class64_regimes_vs_oracle(ctx, mode, lo):
    nmin, nmax = 3000, 7000
    hi = min(lo + 120000, 2**64 - 1)
    p, s0, s1, hits, termsum, _ = run_segment(ctx, mode, nmin, nmax, lo, hi)
    cands = o.candidates(lo, hi)
    assert np.array_equal(p, cands)
    ohits, osum, terms = o.sieve(mode, nmin, nmax, cands, THREADS, want_terms=True)
    assert np.array_equal(s0, terms[:, 0])
    if mode == 5:
        assert np.array_equal(s1, terms[:, 2])
    assert np.array_equal(hits, ohits)
    assert termsum == osum


@pytest.mark.parametrize("nmin,nmax,pmin,pmax", [
    (101, 5000, 10**6, 10**6 + 10**4),                  # class-32 words
    (3000, 7000, 2**40, 2**40 + 10**4),                  # 128-bit words
    (3000, 7000, 2**63, 2**63 + 10**4),                  # 64-bit words
    (2_000_000, 2_000_100, 10**9, 2**33),                # two forms, large n0
    (101, 102, 2**31 - 10**4, LAZY_END + 10**4),         # all three forms
])
@pytest.mark.parametrize("mode", [1, 2, 4, 5])
def test_table_self_check(ctx, mode, nmin, nmax, pmin, pmax):
    """Every setup-program form the job built, run by the setup kernel on a
    test prime, equals the slow products; walk tables match by product and
    count."""
    with pfc.Job(ctx, mode, nmin, nmax, pmin, pmax) as job:
        assert job.verify_tables() > 0


def test_wilson_and_small_p(ctx):
    """p <= n: residues fall to 0 and (p-1)!+1 hits are real (self-test 3/6/10/14)."""
    for mode in (1, 2, 4, 5):
        p, s0, s1, hits, termsum, _ = run_segment(ctx, mode, 101, 6000, 3, 6000)
        cands = o.candidates(3, 6000)
        ohits, osum, terms = o.sieve(mode, 101, 6000, cands, THREADS, want_terms=True)
        assert np.array_equal(s0, terms[:, 0]) and np.array_equal(hits, ohits) and termsum == osum


# --------------------------------------------------- stage API, chunking

@pytest.mark.parametrize("mode", [1, 2, 4, 5])
def test_uneven_iterate_chunks(ctx, mode):
    nmin, nmax, pmin, pmax = 150, 9001, 10**6, 10**6 + 40000
    cands = o.candidates(pmin, pmax)
    ohits, osum, terms = o.sieve(mode, nmin, nmax, cands, THREADS, want_terms=True)
    with pfc.Job(ctx, mode, nmin, nmax, pmin, pmax) as job:
        job.gen(pmin, pmax)
        job.setup()
        cuts = [nmin, nmin + 1, nmin + 8, nmin + 9, nmin + 40, 3001, 3017, 7000, nmax]
        for a, b in zip(cuts[:-1], cuts[1:]):
            job.iterate(a, b)
        job.check()
        p, s0, s1 = job.segment_state()
        hits = o.sort_factors(job.drain_hits())
        termsum, _ = job.totals()
    order = np.argsort(p)
    assert np.array_equal(s0[order], terms[:, 0])
    assert np.array_equal(hits, ohits)
    assert termsum == osum


def test_out_of_order_iterate_rejected(ctx):
    with pfc.Job(ctx, 1, 101, 1000, 10**6, 10**6 + 1000) as job:
        job.gen(10**6, 10**6 + 1000)
        with pytest.raises(pfc.PFCError):
            job.iterate(101, 200)   # before setup
        job.setup()
        with pytest.raises(pfc.PFCError):
            job.iterate(200, 300)   # skips [101, 200)
        with pytest.raises(pfc.PFCError):
            job.check()             # n range incomplete


def test_segment_split_invariance(ctx):
    """Totals over a p range equal the sum over any split of it."""
    mode, nmin, nmax = 5, 101, 20000
    lo, hi = 10**8, 10**8 + 400000
    with pfc.Job(ctx, mode, nmin, nmax, lo, hi) as job:
        job.segment(lo, hi)
        whole = job.totals()
        h1 = o.sort_factors(job.drain_hits())
    with pfc.Job(ctx, mode, nmin, nmax, lo, hi) as job:
        for a, b in [(lo, lo + 123457), (lo + 123457, lo + 300001), (lo + 300001, hi)]:
            job.segment(a, b)
        split = job.totals()
        h2 = o.sort_factors(job.drain_hits())
    assert whole == split
    assert np.array_equal(h1, h2)


# ------------------------------------------- the reference's self-test

@pytest.mark.parametrize("cid", list(range(1, 17)))
def test_selftest_triple(ctx, cid):
    c = goldens.case(cid)
    r = pfc.sieve(c["mode"], c["nmin"], c["nmax"], c["pmin"], c["pmax"], threads=THREADS, ctx=ctx)
    assert (r.factorcount, r.primecount, r.checksum) == (c["factors"], c["primecount"], c["checksum_int"])


@pytest.mark.parametrize("cid", [3, 9, 10, 14])
def test_selftest_factor_lists(ctx, cid):
    """Whole factor lists (not just the triple) equal the oracle's."""
    c = goldens.case(cid)
    r = pfc.sieve(c["mode"], c["nmin"], c["nmax"], c["pmin"], c["pmax"], threads=THREADS, ctx=ctx)
    _, ofac = o.job(c["mode"], c["nmin"], c["nmax"], c["pmin"], c["pmax"], THREADS)
    assert np.array_equal(o.sort_factors(r.factors), o.sort_factors(ofac))


# ---------------------------------------------- walk variants (autotuning)

@pytest.mark.parametrize("cls,lo", [(0, 10**9), (1, 2**40)])
def test_every_walk_variant_vs_oracle(cls, lo):
    """Each compiled walk variant (candidates per thread, block length) gives
    the oracle's residues, hits and checksum terms, in every mode."""
    hi = lo + 300000
    cands = o.candidates(lo, hi)
    with pfc.Context(0) as c:
        for fused in (0, 1):
            modes = [5] if fused else [1, 2, 4]
            nvar = {(0, 0): 3, (0, 1): 2, (1, 0): 2, (1, 1): 2}[(cls, fused)]
            for mode in modes:
                ohits, osum, terms = o.sieve(mode, 3000, 7001, cands, THREADS, want_terms=True)
                for v in range(nvar):
                    c.set_walk_variant(cls, fused, v)
                    p, s0, s1, hits, termsum, _ = run_segment(c, mode, 3000, 7001, lo, hi)
                    assert np.array_equal(s0, terms[:, 0]), (mode, v)
                    if mode == 5:
                        assert np.array_equal(s1, terms[:, 2]), v
                    assert np.array_equal(hits, ohits), (mode, v)
                    assert termsum == osum, (mode, v)


def test_autotune_reports_and_picks_one_variant_per_kind():
    with pfc.Context(0) as c:
        rep = c.autotune()
        lines = [x for x in rep.splitlines() if x]
        # class 32 single (3 variants) and fused (2), lazy class 64 single (4) and fused (2)
        assert len(lines) == 3 + 2 + 4 + 2
        for kind in ("class32 single", "class32 fused", "class64-lazy single", "class64-lazy fused"):
            assert sum(1 for x in lines if x.startswith(kind) and x.endswith("*")) == 1
        v, nc, b = c.walk_variant(0, 0)
        assert (nc, b) in ((2, 16), (2, 8), (1, 16))
        v, nc, b = c.walk_variant(1, 0)
        assert (nc, b) in ((1, 32), (1, 16), (1, 8), (2, 16))


@pytest.mark.parametrize("mode", [1, 2, 4, 5])
def test_segment_graphs_equal_stream_launches(mode):
    """Several segments of one job replayed as a CUDA graph (re-captured when
    the candidate buffers grow and at the class-64 boundary) give the same
    totals and hits as the same launches issued on the stream."""
    lo, hi = 2**31 - 400000, 2**31 + 600000
    cuts = [lo, lo + 100000, lo + 130000, lo + 400000, 2**31 + 1, 2**31 + 300000, hi]
    out = []
    for graphs in (False, True):
        with pfc.Context(0) as c:
            c.set_graphs(graphs)
            with pfc.Job(c, mode, 2000, 9000, lo, hi) as job:
                for a, b in zip(cuts[:-1], cuts[1:]):
                    job.segment(a, b)
                out.append((job.totals(), o.sort_factors(job.drain_hits())))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])


# split walks: (mode, nmin, nmax, p_lo, p_hi) with few candidates and a small
# nmin, so that the n range is cut into sub-ranges; every size class, both
# classes in one segment, the fused walk and the primorial's prime indices
SPLIT_CASES = [
    (1, 101, 20000, 10**7, 10**7 + 200000),
    (5, 101, 30000, 10**9, 10**9 + 300000),
    (4, 101, 30000, 10**9, 10**9 + 300000),
    (2, 101, 200000, 2**62, 2**62 + 300000),
    (5, 200, 30000, 2**40, 2**40 + 300000),
    (1, 101, 20000, 2**64 - 600000, 2**64 - 1),
    (1, 101, 20000, 2**31 - 200000, 2**31 + 200000),
    (1, 101, 20000, 3, 60000),
]


def split_run(case, split, stage_calls=False):
    mode, nmin, nmax, lo, hi = case
    with pfc.Context(0) as c:
        c.set_split(split)
        with pfc.Job(c, mode, nmin, nmax, lo, hi) as job:
            l0 = c.launches
            if stage_calls:
                job.gen(lo, hi)
                job.setup()
                job.iterate(nmin, nmax)
                job.check()
            else:
                job.segment(lo, hi)
            launches = c.launches - l0
            p, s0, s1 = job.segment_state()
            order = np.argsort(p)
            return (job.totals(), o.sort_factors(job.drain_hits()), p[order], s0[order], s1[order], launches)


@pytest.mark.parametrize("case", SPLIT_CASES)
def test_split_walk_equals_the_plain_walk(case):
    """The walk cut into n sub-ranges (start residues from setup programs)
    leaves the same residues, totals and hits as one chain per candidate;
    it did run split (its extra setup launches)."""
    plain = split_run(case, False)
    split = split_run(case, True)
    assert split[5] > plain[5], "the split walk did not run"
    assert split[0] == plain[0]
    assert np.array_equal(split[1], plain[1])
    for k in (2, 3, 4):
        assert np.array_equal(split[k], plain[k])


@pytest.mark.parametrize("case", [SPLIT_CASES[0], SPLIT_CASES[1], SPLIT_CASES[3]])
def test_split_walk_through_the_stage_calls(case):
    """pfc_iterate over the whole range walks split too, with the same result
    as the plain walk through pfc_segment."""
    plain = split_run(case, False)
    staged = split_run(case, True, stage_calls=True)
    assert staged[0] == plain[0]
    assert np.array_equal(staged[1], plain[1])
    assert np.array_equal(staged[3], plain[3]) and np.array_equal(staged[4], plain[4])


def test_split_walk_matches_the_oracle():
    """Hits and residues of a split walk against the oracle directly."""
    mode, nmin, nmax, lo, hi = SPLIT_CASES[1]
    totals, hits, p, s0, s1, _ = split_run(SPLIT_CASES[1], True)
    cands = o.candidates(lo, hi)
    assert np.array_equal(p, cands)
    ohits, _, terms = o.sieve(mode, nmin, nmax, cands, want_terms=True)
    assert np.array_equal(s0, terms[:, 0]) and np.array_equal(s1, terms[:, 2])
    assert np.array_equal(hits, ohits)


# tensor-core setup (class 64 below 2^64/3): programs of one tile and of many
# (group boundaries inside tiles), both programs of the combined search, a
# product program without squarings, p just above 2^31 and near 2^64/3
# programs at or above the tensor-core thresholds (kernels.cuh: 480 words in
# class 64, 448 in class 32; smaller ones keep the integer setup)
TC_CASES = [
    (1, 400000, 400100, 2**40, 2**40 + 20000),          # 910 words
    (1, 500000, 500100, 2**50, 2**50 + 20000),          # 1138
    (5, 300000, 300050, 2**62, 2**62 + 20000),          # 895
    (2, 600000, 600050, 2**31 + 10, 2**31 + 40000),     # 975
    (4, 600000, 600050, 6 * 10**18, 6 * 10**18 + 40000),   # 805
    # class 32 (four byte planes, 64 candidates per CTA), and both classes in one segment
    (1, 400000, 400100, 10**9, 10**9 + 200000),         # 910
    (5, 300000, 300050, 2**31 - 40000, 2**31 - 10),     # 895
    (2, 400000, 400100, 10**7, 10**7 + 200000),         # 650
    (4, 600000, 600100, 2**31 - 100000, 2**31 + 100000),   # 805
    # just above the thresholds
    (1, 210000, 210100, 2**40, 2**40 + 20000),          # 483
    (1, 200000, 200100, 10**9, 10**9 + 200000),         # 460
    # below the thresholds: the integer setup, through the same switch
    (1, 20000, 20100, 2**40, 2**40 + 20000),            # 56
    (1, 40000, 40100, 10**9, 10**9 + 200000),           # 101
    (1, 200000, 200100, 2**40, 2**40 + 20000),          # 460 (class 64)
    (1, 190000, 190100, 10**9, 10**9 + 200000),         # 439 (class 32)
]


def setup_run(case, tc):
    mode, nmin, nmax, lo, hi = case
    with pfc.Context(0) as c:
        c.set_setup_tc(tc)
        c.set_split(False)
        with pfc.Job(c, mode, nmin, nmax, lo, hi) as job:
            job.segment(lo, hi)
            p, s0, s1 = job.segment_state()
            order = np.argsort(p)
            return job.totals(), o.sort_factors(job.drain_hits()), p[order], s0[order], s1[order]


@pytest.mark.parametrize("case", TC_CASES)
def test_tensor_core_setup_equals_the_integer_setup(case):
    tc = setup_run(case, True)
    ip = setup_run(case, False)
    assert tc[0] == ip[0]
    assert np.array_equal(tc[1], ip[1])
    for k in (2, 3, 4):
        assert np.array_equal(tc[k], ip[k])


@pytest.mark.parametrize("case", [TC_CASES[2], TC_CASES[6]])
def test_tensor_core_setup_matches_the_oracle(case):
    mode, nmin, nmax, lo, hi = case
    totals, hits, p, s0, s1 = setup_run(case, True)
    cands = o.candidates(lo, hi)
    assert np.array_equal(p, cands)
    ohits, _, terms = o.sieve(mode, nmin, nmax, cands, want_terms=True)
    assert np.array_equal(s0, terms[:, 0]) and np.array_equal(s1, terms[:, 2])
    assert np.array_equal(hits, ohits)
