"""C ABI checks that need no GPU: the library builds and loads, exports every
symbol include/pfcsieve.h declares, and its host-side routines (factor
post-processing, primality, formatting, status strings) match the oracle and
the reference's formats."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle as o

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def pfc():
    from pfcsieve_gb300 import build
    build.build()
    import pfcsieve_gb300
    pfcsieve_gb300.lib()
    return pfcsieve_gb300


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(pfc_\w+)\s*\(", txt))
    return names


def test_exports_every_declared_symbol(pfc):
    L = ctypes.CDLL(pfc.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in sorted(syms):
        assert hasattr(L, s), s


def test_no_device_is_an_error_not_a_fallback(pfc):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(pfc.PFCError) as e:
        pfc.Context(0)
    assert e.value.code == pfc.PFC_ERR_NO_DEVICE


def test_status_strings(pfc):
    for code in range(-10, 1):
        assert pfc.status_string(code) != "unknown status"


def test_format_factor_lines(pfc):
    # cl_sieve.cpp:565-581: "%llu | %u!%+d", "%llu | %u#%+d", "%llu | %u!/#%+d"
    assert pfc.format_factor((101, -100, 0)) == "101 | 100!-1"
    assert pfc.format_factor((1000000007, 12345, 1)) == "1000000007 | 12345#+1"
    assert pfc.format_factor((18446744073709551557, -2147483647, 2)) == \
        "18446744073709551557 | 2147483647!/#-1"


def test_is_prime_matches_oracle(pfc):
    rng = np.random.default_rng(3)
    xs = list(range(1, 5000)) + [42799, 85489, 4294967297, 3215031751, 2152302898747,
                                 3474749660383, 341550071728321, 3825123056546413051,
                                 18446744073709551557, 18446744073709551615]
    xs += [int(x) | 1 for x in rng.integers(1, 2**63, size=3000, dtype=np.uint64)]
    for x in xs:
        assert pfc.is_prime(x) == o.is_prime(x), x


def test_is_prime_below_2_32_matches_oracle(pfc):
    """Below 2^32 the host test takes three 32-bit bases: its verdicts equal
    the reference's seven-base test (the oracle) on dense windows at 2^31
    and below 2^32, random 32-bit values, and every base-2 strong
    pseudoprime under 10^6 (they pass the first base)."""
    rng = np.random.default_rng(5)
    xs = list(range(2**31 - 20001, 2**31 + 20001, 2)) + list(range(2**32 - 40001, 2**32, 2))
    xs += [int(x) | 1 for x in rng.integers(3, 2**32, size=20000, dtype=np.uint64)]
    spsp = [x for x in range(3, 10**6, 2) if o.strong_prp_two(x) and not o.is_prime(x)]
    assert 2047 in spsp and len(spsp) > 40
    xs += spsp + [3215031751, 4759123141, 2**32 - 5, 2**32 + 15]
    for x in xs:
        assert pfc.is_prime(x) == o.is_prime(x), x


@pytest.mark.parametrize("mode,nmin,nmax,pmin,pmax", [
    (1, 101, 200000, 101, 20000), (2, 101, 200000, 101, 20000),
    (4, 101, 200000, 101, 20000), (5, 101, 50000, 3, 30000),
])
def test_finalize_matches_oracle_job(pfc, mode, nmin, nmax, pmin, pmax):
    """pfc_finalize_factors on the oracle's raw hits reproduces the oracle's
    whole-job factor list and checksum (sort, CPU verify, 2-PRP drop, fold)."""
    cands = o.candidates(pmin, pmax)
    hits, termsum, _ = o.sieve(mode, nmin, nmax, cands, os.cpu_count() or 1)
    res, ofac = o.job(mode, nmin, nmax, pmin, pmax, os.cpu_count() or 1)
    kept, add = pfc.finalize(mode, nmax, hits[::-1].copy(), threads=4, verify=True)
    assert (termsum + add) % 2**64 == res.checksum
    assert np.array_equal(o.sort_factors(kept), o.sort_factors(ofac))


@pytest.mark.parametrize("p", [1000003, 16777259, 33554467])
def test_finalize_accepts_wilson_hits_over_long_ranges(pfc, p):
    """(p-1)! = -1 (mod p) (Wilson): the record (p, +(p-1), factorial) is a
    true hit and the other sign is not; the re-verification walks up to 3.4e7
    consecutive terms (the block-product path)."""
    assert o.is_prime(p)
    rec = np.zeros(1, dtype=pfc.FACTOR_DTYPE)
    rec[0] = (p, p - 1, 0)
    kept, _ = pfc.finalize(1, 2**31 - 1, rec, threads=1)
    assert len(kept) == 1
    rec[0] = (p, -(p - 1), 0)
    with pytest.raises(pfc.PFCError):
        pfc.finalize(1, 2**31 - 1, rec, threads=1)


def test_finalize_accepts_true_hits_above_2_32(pfc):
    """True hits of every type with p above 2^32 (the 64-bit arithmetic of
    the re-verification), found by the oracle (tests/golden/make_verify_hits.py):
    all are kept, and copies with the sign flipped, n moved by one or p moved
    to the next odd number fail as the reference's check would fail them."""
    d = np.load(os.path.join(ROOT, "tests", "golden", "verify_hits_64.npz"))
    types = set()
    for i in range(2):
        mode, nmin, nmax, pmin, pmax = [int(x) for x in d["s%d_params" % i]]
        hits = d["s%d_hits" % i]
        assert len(hits) > 10 and (hits["p"] > 2**32).all()
        types |= set(int(t) for t in hits["type"])
        kept, add = pfc.finalize(mode, nmax, hits.copy(), threads=2)
        assert len(kept) == len(hits)
        assert add == sum(abs(int(x)) + (1 if x > 0 else -1) for x in hits["nc"]) % 2**64
        for r in hits:
            flipped = np.array([r], dtype=pfc.FACTOR_DTYPE)
            flipped["nc"] = -flipped["nc"]
            with pytest.raises(pfc.PFCError):
                pfc.finalize(mode, nmax, flipped, threads=1)
    assert types == {0, 1, 2}


@pytest.mark.parametrize("name", ["cfg1", "cfg2"])
def test_finalize_keeps_the_reference_programs_factors(pfc, name):
    """The factors.txt the reference's own OpenCL program wrote for two
    benchmark searches (tests/golden/ref_opencl_*_factors.txt), read back as
    records: the host re-verification and 2-PRP filter keep every one, and
    they format to the same lines (cl_sieve.cpp:565-581)."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "configs.npz"))
    mode, nmin, nmax = (int(x) for x in g[name + "_params"][:3])
    lines = open(os.path.join(ROOT, "tests", "golden", "ref_opencl_%s_factors.txt" % name)).read().splitlines()
    body = [x for x in lines[:-1] if x != "no factors"]
    recs = np.zeros(len(body), dtype=pfc.FACTOR_DTYPE)
    for i, line in enumerate(body):
        ps, rest = line.split(" | ")
        m = re.match(r"(\d+)(!/#|!|#)([+-]1)$", rest)
        n, typ, c = int(m.group(1)), {"!": 0, "#": 1, "!/#": 2}[m.group(2)], int(m.group(3))
        recs[i] = (int(ps), c * n if c > 0 else -n, typ)
    kept, add = pfc.finalize(mode, nmax, recs.copy(), threads=4)
    assert len(kept) == len(body) > 200
    assert add == sum(abs(int(x)) + (1 if x > 0 else -1) for x in recs["nc"]) % 2**64
    assert sorted(pfc.format_factor(f) for f in kept) == sorted(body)


def test_finalize_rejects_false_hit(pfc):
    bad = np.zeros(1, dtype=pfc.FACTOR_DTYPE)
    bad[0] = (1000003, -1000, 0)   # 1000003 does not divide 1000!-1
    with pytest.raises(pfc.PFCError) as e:
        pfc.finalize(1, 2000, bad, verify=True)
    assert e.value.code == -6


@pytest.mark.parametrize("mode", [1, 2, 4])
def test_finalize_rejects_flipped_sign(pfc, mode):
    """A true hit with its sign flipped (p divides n!+1, reported as n!-1) fails
    the CPU verification in every walk type, at the largest n of the hits
    (the longest verification product)."""
    nmin, nmax, pmin, pmax = 101, 30000, 101, 20000
    hits, _, _ = o.sieve(mode, nmin, nmax, o.candidates(pmin, pmax), os.cpu_count() or 1)
    assert len(hits)
    kept, _ = pfc.finalize(mode, nmax, hits.copy(), threads=4, verify=True)
    bad = hits.copy()
    i = int(np.argmax(np.abs(bad["nc"])))
    bad["nc"][i] = -bad["nc"][i]
    with pytest.raises(pfc.PFCError) as e:
        pfc.finalize(mode, nmax, bad, threads=4, verify=True)
    assert e.value.code == -6


def _program_model(mode, nmin):
    """Setup program size from the definition: (nmin-1)! (mode 1), its
    composite part (mode 4) or the primorial (mode 2) as prime products
    grouped by the bits of the Legendre exponents (Horner form: one squaring
    between consecutive bit levels), each group packed greedily into 896-bit
    words two primes at a time, then one; mode 5 = mode 4 + the primorial."""
    n0 = nmin - 1
    primes = [q for q in range(2, n0 + 1) if all(q % d for d in range(2, int(q ** 0.5) + 1))]

    def pack(fs):
        words, i = 0, 0
        while i < len(fs):
            acc = fs[i]
            i += 1
            while i < len(fs):
                for take in ((2, 1) if i + 1 < len(fs) else (1,)):
                    m = fs[i] * fs[i + 1] if take == 2 else fs[i]
                    if (acc * m).bit_length() <= 896:
                        acc *= m
                        i += take
                        break
                else:
                    break
            words += 1
        return words

    def power(sub):
        bits = {}
        for q in primes:
            e, qk = 0, q
            while qk <= n0:
                e += n0 // qk
                qk *= q
            e -= sub
            j = 0
            while e:
                if e & 1:
                    bits.setdefault(j, []).append(q)
                e >>= 1
                j += 1
        if not bits:
            return 0, 0
        top = max(bits)
        return sum(pack(bits[j]) for j in bits), top

    if mode == 1:
        return power(0)
    if mode == 2:
        return pack(primes), 0
    w, s = power(1)
    return (w + pack(primes), s) if mode == 5 else (w, s)


@pytest.mark.parametrize("mode,nmin", [(1, 101), (1, 5000), (2, 5000), (4, 5000), (5, 20011), (1, 65537)])
def test_setup_program_size_matches_the_definition(pfc, mode, nmin):
    assert pfc.setup_program_size(mode, nmin) == _program_model(mode, nmin)


def _start_residues(nmin, ps):
    """(n-1)!, (n-1)# and (n-1)!/(n-1)# mod each p, n = nmin: the starting
    residues the reference's setup computes (kernels/setup.cl:49-288), from
    their definition."""
    N = nmin - 1
    isp = np.ones(N + 1, dtype=bool)
    isp[:2] = False
    for i in range(2, int(N ** 0.5) + 1):
        if isp[i]:
            isp[i * i::i] = False
    out = {}
    for p in ps:
        f = pr = c = 1
        for n in range(2, N + 1):
            f = f * n % p
            if isp[n]:
                pr = pr * n % p
            else:
                c = c * n % p
        out[p] = (f, pr, c)
    return out


# programs below and above the tensor-core setup's thresholds (kTcMinWords32/64):
# 7, 214 and 460 896-bit words for the factorial
@pytest.mark.parametrize("nmin", [101, 90001, 200001])
def test_setup_programs_replayed_on_the_host_give_the_start_residues(pfc, nmin):
    """Every form of the host-built setup programs -- 64-bit words, 896-bit
    words, and the tensor-core setup's pairs of 896-bit words with their own
    groups and power-of-R correction -- replayed as the device runs them
    gives the definition's starting residues, for p in every size class and a
    composite candidate (a base-2 pseudoprime)."""
    ps = [int(o.candidates(10**9, 10**9 + 200)[0]), 2**31 - 1, int(o.candidates(2**40, 2**40 + 200)[0]),
          int(o.candidates(2**62, 2**62 + 400)[0]), 2**64 - 59, 4294967297]
    want = _start_residues(nmin, ps)
    for p in ps:
        f, pr, c = want[p]
        for form in ("narrow", "wide", "paired"):
            assert pfc.setup_program_eval(1, nmin, p, form) == (f, 0), (p, form)
            assert pfc.setup_program_eval(2, nmin, p, form) == (pr, 0), (p, form)
            assert pfc.setup_program_eval(4, nmin, p, form) == (c, 0), (p, form)
            assert pfc.setup_program_eval(5, nmin, p, form) == (f, c), (p, form)


def test_setup_program_eval_rejects_bad_arguments(pfc):
    for mode, nmin, p in [(3, 101, 10**9 + 7), (1, 100, 10**9 + 7), (1, 101, 10**9 + 8), (1, 101, 1)]:
        with pytest.raises(pfc.PFCError):
            pfc.setup_program_eval(mode, nmin, p)
