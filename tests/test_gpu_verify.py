"""Device re-verification of hits (pfc_verify_factors_device) against the CPU
check that the reference runs (pfc_finalize_factors with verify, the check of
verifyprime.cpp:199-268), which remains the check of record.

Bar: the device's verdict equals the CPU check's verdict hit by hit, on true
hits of every walk type and on records with one field wrong (sign, n, p), and
finalize(verify="device") returns exactly what finalize(verify=True) returns.
All tests need a GB300 (marker gpu).
"""
import os

import numpy as np
import pytest

from oracle import oracle as o

pfc = pytest.importorskip("pfcsieve_gb300")

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def ctx():
    c = pfc.Context(0)
    yield c
    c.close()


def cpu_verdicts(mode, nmax, recs):
    """The CPU check one record at a time: True where it fails."""
    out = []
    for r in recs:
        try:
            pfc.finalize(mode, nmax, np.array([r], dtype=pfc.FACTOR_DTYPE), threads=1, verify=True)
            out.append(False)
        except pfc.PFCError as e:
            assert e.code == -6
            out.append(True)
    return np.array(out)


def damaged(hits, rng, count):
    """Copies of true hits with one field changed: the sign, n by one, or p
    moved to the next odd number."""
    recs = hits.copy()
    pick = rng.choice(len(recs), size=min(count, len(recs)), replace=False)
    for j, i in enumerate(pick):
        kind = j % 3
        if kind == 0:
            recs["nc"][i] = -recs["nc"][i]
        elif kind == 1:
            recs["nc"][i] += 1 if recs["nc"][i] > 0 else -1
        else:
            recs["p"][i] += 2
    return recs, pick


@pytest.mark.parametrize("mode,nmin,nmax,pmin,pmax", [
    (1, 101, 30000, 101, 20000), (2, 101, 200000, 101, 20000),
    (4, 101, 50000, 101, 20000), (5, 101, 30000, 3, 20000),
])
def test_device_verdicts_equal_the_cpu_check(ctx, mode, nmin, nmax, pmin, pmax):
    hits, _, _ = o.sieve(mode, nmin, nmax, o.candidates(pmin, pmax), THREADS)
    assert len(hits)
    assert not pfc.verify_factors(ctx, mode, nmax, hits).any()
    rng = np.random.default_rng(mode)
    recs, pick = damaged(hits, rng, 24)
    dev = pfc.verify_factors(ctx, mode, nmax, recs)
    cpu = cpu_verdicts(mode, nmax, recs)
    assert np.array_equal(dev, cpu)
    assert dev[pick[0::3]].all()   # a flipped sign always fails (n +- 1 can pass a primorial check)
    kept_c, add_c = pfc.finalize(mode, nmax, hits, threads=THREADS, verify=True)
    kept_d, add_d = pfc.finalize(mode, nmax, hits, threads=THREADS, verify="device", ctx=ctx)
    assert add_c == add_d and np.array_equal(kept_c, kept_d)


@pytest.mark.parametrize("mode,nmin,nmax,pmin,pmax", [
    (1, 1000000, 1020000, 10**9, 10**9 + 2 * 10**8),
    (4, 1000000, 1030000, 10**9, 10**9 + 2 * 10**8),
    (2, 300000, 2000000, 2**33, 2**33 + 2 * 10**8),
])
def test_large_n_hits_of_a_gpu_search(ctx, mode, nmin, nmax, pmin, pmax):
    """Hits at n near 10^6 (products of 10^6 terms per hit) from the GPU
    sieve itself: both checks pass them, both reject them with a flipped sign."""
    with pfc.Job(ctx, mode, nmin, nmax, pmin, pmax) as job:
        hits = job.run()
    assert len(hits) > 0
    assert not pfc.verify_factors(ctx, mode, nmax, hits).any()
    pfc.finalize(mode, nmax, hits, threads=THREADS, verify=True)
    bad = hits.copy()
    bad["nc"] = -bad["nc"]
    assert pfc.verify_factors(ctx, mode, nmax, bad).all()
    assert cpu_verdicts(mode, nmax, bad[:4]).all()


def test_sieve_with_device_verification(ctx):
    want = pfc.sieve(5, 101, 20000, 10**9, 10**9 + 10**7, threads=THREADS, ctx=ctx)
    got = pfc.sieve(5, 101, 20000, 10**9, 10**9 + 10**7, threads=THREADS, ctx=ctx, verify="device")
    assert (got.factorcount, got.primecount, got.checksum) == (want.factorcount, want.primecount, want.checksum)
    assert np.array_equal(got.factors, want.factors)


def test_empty_and_invalid_records(ctx):
    assert len(pfc.verify_factors(ctx, 1, 1000, np.zeros(0, dtype=pfc.FACTOR_DTYPE))) == 0
    rec = np.zeros(1, dtype=pfc.FACTOR_DTYPE)
    rec[0] = (1000003, -500, 7)   # no such walk type
    with pytest.raises(pfc.PFCError) as e:
        pfc.verify_factors(ctx, 1, 1000, rec)
    assert e.value.code == -1
    rec[0] = (1000004, -500, 0)   # even p
    with pytest.raises(pfc.PFCError) as e:
        pfc.verify_factors(ctx, 1, 1000, rec)
    assert e.value.code == -1
