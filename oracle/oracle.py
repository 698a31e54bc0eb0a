"""ctypes wrapper around the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  The product (pfcsieve_gb300) never loads it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libpfcref.so")

FACTORIAL, PRIMORIAL, COMPOSITORIAL = 1, 2, 4

FACTOR_DTYPE = np.dtype([("p", "<u8"), ("nc", "<i4"), ("type", "<i4")])


class OrcResult(ctypes.Structure):
    _fields_ = [
        ("checksum", ctypes.c_uint64),
        ("primecount", ctypes.c_uint64),
        ("factorcount", ctypes.c_uint64),
        ("hitcount", ctypes.c_uint64),
        ("pairs", ctypes.c_uint64),
    ]


def build(force=False):
    """Compile liboracle.so (and oracle/_ref when the reference is present)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u64, u32, i32 = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32
        vp = ctypes.c_void_p
        L.orc_invert.restype = u64
        L.orc_invert.argtypes = [u64]
        L.orc_m_mul.restype = u64
        L.orc_m_mul.argtypes = [u64, u64, u64, u64]
        L.orc_add.restype = u64
        L.orc_add.argtypes = [u64, u64, u64]
        L.orc_strong_prp_two.restype = ctypes.c_int
        L.orc_strong_prp_two.argtypes = [u64]
        L.orc_is_prime.restype = ctypes.c_int
        L.orc_is_prime.argtypes = [u64]
        L.orc_verify.restype = ctypes.c_int
        L.orc_verify.argtypes = [u64, u32, i32, i32, vp, ctypes.c_size_t]
        L.orc_candidates.restype = u64
        L.orc_candidates.argtypes = [u64, u64, vp, u64]
        L.orc_sieve.restype = ctypes.c_int
        L.orc_sieve.argtypes = [ctypes.c_uint, u32, u32, vp, u64, ctypes.c_int,
                                vp, u64, ctypes.POINTER(u64), ctypes.POINTER(u64), vp]
        L.orc_job.restype = ctypes.c_int
        L.orc_job.argtypes = [ctypes.c_uint, u32, u32, u64, u64, ctypes.c_int,
                              vp, u64, ctypes.POINTER(OrcResult)]
        L.orc_primes_range.restype = u64
        L.orc_primes_range.argtypes = [u32, u32, vp, u64]
        _lib = L
    return _lib


def candidates(pmin, pmax):
    L = lib()
    n = L.orc_candidates(pmin, pmax, None, 0)
    out = np.zeros(max(n, 1), dtype=np.uint64)
    L.orc_candidates(pmin, pmax, out.ctypes.data, n)
    return out[:n]


def primes_range(lo, hi):
    L = lib()
    n = L.orc_primes_range(lo, hi, None, 0)
    out = np.zeros(max(n, 1), dtype=np.uint32)
    L.orc_primes_range(lo, hi, out.ctypes.data, n)
    return out[:n]


def sieve(mode, nmin, nmax, cands, threads=0, want_terms=False):
    """setup+iterate+check for explicit candidates.

    Returns (hits[sorted], termsum, terms or None); terms rows are
    (s6, s7, s4, term) per candidate in input order.
    """
    L = lib()
    cands = np.ascontiguousarray(cands, dtype=np.uint64)
    cap = 1 << 12
    terms = np.zeros((len(cands), 4), dtype=np.uint64) if want_terms else None
    while True:
        hits = np.zeros(cap, dtype=FACTOR_DTYPE)
        nh = ctypes.c_uint64(0)
        ts = ctypes.c_uint64(0)
        rc = L.orc_sieve(mode, nmin, nmax, cands.ctypes.data, len(cands), threads,
                         hits.ctypes.data, cap, ctypes.byref(nh), ctypes.byref(ts),
                         terms.ctypes.data if terms is not None else None)
        if rc:
            raise RuntimeError("orc_sieve failed: %d" % rc)
        if nh.value <= cap:
            break
        cap = nh.value
    hits = sort_factors(hits[: nh.value])
    return hits, ts.value, terms


def job(mode, nmin, nmax, pmin, pmax, threads=0):
    """Whole reference job: returns (OrcResult, kept factors sorted)."""
    L = lib()
    cap = 1 << 16
    while True:
        facs = np.zeros(cap, dtype=FACTOR_DTYPE)
        res = OrcResult()
        rc = L.orc_job(mode, nmin, nmax, pmin, pmax, threads, facs.ctypes.data, cap,
                       ctypes.byref(res))
        if rc:
            raise RuntimeError("orc_job failed: %d" % rc)
        if res.factorcount <= cap:
            return res, facs[: res.factorcount]
        cap = res.factorcount


def sort_factors(f):
    """Canonical order: (p, |n|, type, nc)."""
    if len(f) == 0:
        return f
    key = np.lexsort((f["nc"], f["type"], np.abs(f["nc"].astype(np.int64)), f["p"]))
    return f[key]


def m_mul(a, b, p, q):
    return lib().orc_m_mul(a, b, p, q)


def invert(p):
    return lib().orc_invert(p)


def is_prime(p):
    return bool(lib().orc_is_prime(p))


def strong_prp_two(n):
    return bool(lib().orc_strong_prp_two(n))


def power_table(startN):
    L = lib()
    L.orc_power_table.restype = ctypes.c_uint64
    L.orc_power_table.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
    n = L.orc_power_table(startN, None, None, 0)
    prod = np.zeros(max(n, 1), dtype=np.uint64)
    eb = np.zeros(2 * max(n, 1), dtype=np.uint32)
    L.orc_power_table(startN, prod.ctypes.data, eb.ctypes.data, n)
    return prod[:n], eb[: 2 * n]


def prime_products(startN):
    L = lib()
    L.orc_prime_products.restype = ctypes.c_uint64
    L.orc_prime_products.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64]
    n = L.orc_prime_products(startN, None, 0)
    prod = np.zeros(max(n, 1), dtype=np.uint64)
    L.orc_prime_products(startN, prod.ctypes.data, n)
    return prod[:n]


def comp_products(nmin):
    L = lib()
    L.orc_comp_products.restype = ctypes.c_uint64
    L.orc_comp_products.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64]
    n = L.orc_comp_products(nmin, None, 0)
    prod = np.zeros(max(n, 1), dtype=np.uint64)
    L.orc_comp_products(nmin, prod.ctypes.data, n)
    return prod[:n]


# ---------------------------------------------------------------- oracle/_ref

def ref_available():
    """True when oracle/_ref/libpfcref.so (the reference kernels compiled for
    the CPU) exists or can be built from the reference sources here."""
    if not os.path.exists(REF_PATH):
        subprocess.call(["make", "-s", "-C", HERE, "ref"], stdout=subprocess.DEVNULL,
                        stderr=subprocess.DEVNULL)
    return os.path.exists(REF_PATH)


_ref = None


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("oracle/_ref not built (reference sources absent)")
        R = ctypes.CDLL(REF_PATH)
        u64, u32, i32, vp = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32, ctypes.c_void_p
        R.ref_is_prime.restype = ctypes.c_int
        R.ref_is_prime.argtypes = [u64]
        R.ref_verify.restype = ctypes.c_int
        R.ref_verify.argtypes = [u64, u32, i32, i32, vp, ctypes.c_size_t]
        R.ref_m_mul.restype = u64
        R.ref_m_mul.argtypes = [u64, u64, u64, u64]
        R.ref_segment.restype = ctypes.c_int
        R.ref_segment.argtypes = [ctypes.c_uint, u32, u32, vp, u64, vp, vp, u32, vp, u32,
                                  vp, u32, u32, u32, vp, vp, u64, ctypes.POINTER(u64)]
        _ref = R
    return _ref


def ref_segment(mode, nmin, nmax, cands, sstep=7, nstep=997, hit_cap=1 << 22):
    """Run the reference's own setup/iterate kernels (CPU build) over one
    segment.  Returns (records[ncand, 8], hits sorted)."""
    R = ref_lib()
    cands = np.ascontiguousarray(cands, dtype=np.uint64)
    z64 = np.zeros(1, dtype=np.uint64)
    z32 = np.zeros(2, dtype=np.uint32)
    pp, pe, pr, ip = z64, z32, z64, z32
    pc = prc = isz = 0
    if mode & FACTORIAL:
        pp, pe = power_table(nmin - 1)
        pc = len(pp)
    if mode & PRIMORIAL:
        pr = prime_products(nmin - 1)
        prc = len(pr)
        ip = primes_range(nmin, nmax - 1)
        isz = len(ip)
    if mode & COMPOSITORIAL:
        pr = comp_products(nmin)
        prc = len(pr)
        ip = primes_range(nmin, nmax + 320)
        isz = len(ip)
    ip = np.ascontiguousarray(ip, dtype=np.uint32)
    rec = np.zeros((len(cands), 8), dtype=np.uint64)
    hits = np.zeros(hit_cap, dtype=FACTOR_DTYPE)
    nh = ctypes.c_uint64(0)
    rc = R.ref_segment(mode, nmin, nmax, cands.ctypes.data, len(cands),
                       pp.ctypes.data, pe.ctypes.data, pc, pr.ctypes.data, prc,
                       ip.ctypes.data, isz, sstep, nstep,
                       rec.ctypes.data, hits.ctypes.data, hit_cap, ctypes.byref(nh))
    if rc:
        raise RuntimeError("ref_segment failed: %d" % rc)
    return rec, sort_factors(hits[: nh.value])


def ref_terms(mode, rec):
    """Checksum terms from reference records (kernels/check.cl:59,115,161)."""
    with np.errstate(over="ignore"):
        if mode == PRIMORIAL:
            return rec[:, 6].copy()
        if mode == (FACTORIAL | COMPOSITORIAL):
            return rec[:, 4] + rec[:, 6] + rec[:, 7]
        return rec[:, 6] + rec[:, 7]
