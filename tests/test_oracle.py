"""The CPU oracle against the reference's golden vectors (CPU only).

* the reference self-test triples (cl_sieve.cpp:1787-2080) that finish on a
  few CPU cores in seconds; cases 1 and 6 need PFC_SLOW=1 (minutes);
* the committed per-candidate vectors made by the reference's own kernels
  (tests/golden/make_golden.py), and, where the reference sources exist, the
  live reference kernels and verifyprime.cpp;
* the Montgomery primitives against Python integers.
"""
import os
import random

import numpy as np
import pytest

from oracle import oracle as o
from tests import goldens

THREADS = os.cpu_count() or 1


@pytest.mark.parametrize("cid", [3, 9, 10, 14])
def test_selftest_triple(cid):
    c = goldens.case(cid)
    res, facs = o.job(c["mode"], c["nmin"], c["nmax"], c["pmin"], c["pmax"], THREADS)
    assert (res.factorcount, res.primecount, res.checksum) == \
        (c["factors"], c["primecount"], c["checksum_int"])
    assert len(facs) == c["factors"]


@pytest.mark.slow
@pytest.mark.parametrize("cid", [1, 6])
def test_selftest_triple_slow(cid):
    test_selftest_triple(cid)


def test_ref_segments_fixture():
    segs, _, _ = goldens.ref_segments()
    for s in segs:
        cands = o.candidates(s["pmin"], s["pmax"])
        assert np.array_equal(cands, s["cands"])
        hits, termsum, terms = o.sieve(s["mode"], s["nmin"], s["nmax"], cands, THREADS,
                                       want_terms=True)
        ref_terms = goldens.terms_from_records(s["mode"], s["s4s6s7"])
        assert np.array_equal(terms[:, 3], ref_terms), s
        assert np.array_equal(hits, s["hits"]), s


def test_isprime_fixture():
    _, n, v = goldens.ref_segments()
    got = np.array([o.is_prime(int(x)) for x in n], dtype=np.uint8)
    assert np.array_equal(got, v)


def test_live_reference_kernels():
    if not o.ref_available():
        pytest.skip("reference sources not present on this machine")
    # a segment not in the fixture: chunking differs from the oracle's single pass
    cands = o.candidates(2**33 - 5000, 2**33 + 5000)
    for mode in (1, 2, 4, 5):
        rec, rh = o.ref_segment(mode, 700, 2500, cands, sstep=3, nstep=101)
        hits, _, terms = o.sieve(mode, 700, 2500, cands, THREADS, want_terms=True)
        assert np.array_equal(o.ref_terms(mode, rec), terms[:, 3])
        assert np.array_equal(rh, hits)


def test_live_reference_verify():
    if not o.ref_available():
        pytest.skip("reference sources not present on this machine")
    R = o.ref_lib()
    segs, _, _ = goldens.ref_segments()
    import ctypes
    for s in segs[:4]:
        mode = s["mode"]
        lst = None
        if mode & 2:
            lst = o.primes_range(103, s["nmax"])
        elif mode & 4:
            pr = set(o.primes_range(45, s["nmax"]).tolist())
            lst = np.array([n for n in range(45, s["nmax"]) if n not in pr], dtype=np.uint32)
        for h in s["hits"][::7]:
            n, c = abs(int(h["nc"])), (-1 if h["nc"] < 0 else 1)
            t = int(h["type"])
            l = lst if t else None
            ptr = l.ctypes.data if l is not None else None
            size = len(l) if l is not None else 0
            assert R.ref_verify(int(h["p"]), n, c, t, ptr, size) == 1
            assert o.lib().orc_verify(int(h["p"]), n, c, t, ptr, size) == 1


def test_montgomery_primitives():
    rnd = random.Random(5)
    for _ in range(3000):
        bits = rnd.choice([5, 20, 32, 33, 50, 62, 63, 64])
        p = rnd.getrandbits(bits) | 1 | (1 << (bits - 1))
        if p < 3:
            continue
        q = o.invert(p)
        assert (p * q) % 2**64 == 1
        a, b = rnd.randrange(p), rnd.randrange(p)
        assert o.m_mul(a, b, p, q) == (a * b * pow(2**64, -1, p)) % p
        # one operand unreduced (the table words), the other reduced
        w = rnd.getrandbits(64)
        assert o.m_mul(w, b, p, q) == (w * b * pow(2**64, -1, p)) % p


def test_candidates_rule_small():
    """candidate = small prime 3..113, or x >= 114 with no factor <= 113 that is a
    base-2 strong probable prime (getsegprimes.cl:79-223, addsmallprimes.cl)"""
    small = [p for p in range(3, 114) if all(p % d for d in range(2, p))]

    def sprp2(n):
        d, t = n - 1, 0
        while d % 2 == 0:
            d //= 2
            t += 1
        a = pow(2, d, n)
        if a in (1, n - 1):
            return True
        for _ in range(1, t):
            a = a * a % n
            if a == n - 1:
                return True
        return False

    for lo, hi in [(3, 20000), (42700, 42900), (85000, 86000), (2**32 - 3000, 2**32 + 3000),
                   (4294967000, 4294967400)]:
        want = [x for x in range(lo, hi) if (x < 114 and x in small) or
                (x >= 114 and x % 2 and all(x % s for s in small) and sprp2(x))]
        assert o.candidates(lo, hi).tolist() == want
    # the base-2 pseudoprimes 42799 = 127*337 and 85489 = 127*673 are candidates
    assert 42799 in o.candidates(42000, 43000).tolist()
    assert 4294967297 in o.candidates(4294967290, 4294967300).tolist()
