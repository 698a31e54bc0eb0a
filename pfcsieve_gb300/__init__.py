"""pfcsieve_gb300 -- GB300-native (sm_103a) PFCSieve sieve path.

Finds 64-bit primes p dividing n!+-1, n#+-1 or n!/n#+-1 for n in [nmin, nmax)
and p in [pmin, pmax), with the reference's candidate rule, factor list and
checksum.  This module is a thin ctypes binding over the C ABI in
include/pfcsieve.h (libpfcsieve.so, built in-tree by pfcsieve_gb300/build.py).
There is no CPU fallback: without the library or a GB300 every call raises.

    import pfcsieve_gb300 as pfc
    r = pfc.sieve(pfc.FACTORIAL, nmin=101, nmax=20000, pmin=10**7, pmax=11*10**6)
    r.factorcount, r.primecount, r.checksum, r.factors

`sieve()` follows the reference's cl_sieve() (cl_sieve.cpp:1328-1761): the
p range is walked in segments, hits are drained, re-verified on the CPU,
2-PRP factors are dropped and n+-1 of every kept factor joins the checksum.
"""
import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import build as _build

FACTORIAL, PRIMORIAL, COMPOSITORIAL = 1, 2, 4
TYPE_FACTORIAL, TYPE_PRIMORIAL, TYPE_COMPOSITORIAL = 0, 1, 2
FACTOR_DTYPE = np.dtype([("p", "<u8"), ("nc", "<i4"), ("type", "<i4")])

PFC_OK = 0
PFC_ERR_HIT_OVERFLOW = -4
PFC_ERR_NO_DEVICE = -9

LIB_PATH = _build.LIB


BATCH_THROUGHPUT, BATCH_LATENCY = 0, 1


class JobDesc(ctypes.Structure):
    """pfc_job_desc: one search submitted to a batch."""
    _fields_ = [("mode", ctypes.c_uint), ("nmin", ctypes.c_uint32), ("nmax", ctypes.c_uint32),
                ("pmin", ctypes.c_uint64), ("pmax", ctypes.c_uint64)]


class BatchStatus(ctypes.Structure):
    """pfc_batch_status: state and totals of one search in a batch."""
    _fields_ = [("done", ctypes.c_int), ("status", ctypes.c_int), ("term_checksum", ctypes.c_uint64),
                ("primecount", ctypes.c_uint64), ("pairs", ctypes.c_uint64), ("hits", ctypes.c_uint64)]


class BatchTimes(ctypes.Structure):
    """pfc_batch_times: where a batch's time went."""
    _fields_ = [("step_s", ctypes.c_double), ("gpu_s", ctypes.c_double), ("gpu32_s", ctypes.c_double),
                ("gpu64_s", ctypes.c_double), ("prep_s", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("setup_tc_s", ctypes.c_double), ("iterations", ctypes.c_uint64), ("tasks", ctypes.c_uint64)]


class PFCError(RuntimeError):
    def __init__(self, code, where=""):
        self.code = code
        super().__init__("%s: %s (%d)" % (where, status_string(code), code))


_lib = None


def lib():
    """Load libpfcsieve.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libpfcsieve.so not built: run pfcsieve_gb300.build.build() "
                              "(or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        u64, u32, i32, vp, sz = (ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32,
                                 ctypes.c_void_p, ctypes.c_size_t)
        P = ctypes.POINTER
        sig = {
            "pfc_ctx_create": (ctypes.c_int, [ctypes.c_int, u64, P(vp)]),
            "pfc_ctx_destroy": (ctypes.c_int, [vp]),
            "pfc_ctx_stream": (vp, [vp]),
            "pfc_ctx_launch_count": (u64, [vp]),
            "pfc_ctx_transfer_bytes": (ctypes.c_int, [vp, P(u64), P(u64)]),
            "pfc_ctx_device_info": (ctypes.c_int, [vp, ctypes.c_char_p, sz, P(ctypes.c_int)]),
            "pfc_job_create": (ctypes.c_int, [vp, ctypes.c_uint, u32, u32, u64, u64, P(vp)]),
            "pfc_job_destroy": (ctypes.c_int, [vp]),
            "pfc_job_segment_end": (ctypes.c_int, [vp, u64, P(u64)]),
            "pfc_gen_candidates": (ctypes.c_int, [vp, u64, u64]),
            "pfc_setup": (ctypes.c_int, [vp]),
            "pfc_iterate": (ctypes.c_int, [vp, u32, u32]),
            "pfc_check": (ctypes.c_int, [vp]),
            "pfc_segment": (ctypes.c_int, [vp, u64, u64]),
            "pfc_sync": (ctypes.c_int, [vp]),
            "pfc_drain_hits": (ctypes.c_int, [vp, vp, sz, P(sz)]),
            "pfc_job_totals": (ctypes.c_int, [vp, P(u64), P(u64)]),
            "pfc_job_run": (ctypes.c_int, [vp, vp, sz, P(sz)]),
            "pfc_segment_state": (ctypes.c_int, [vp, vp, vp, vp, sz, P(sz)]),
            "pfc_job_pairs": (u64, [vp]),
            "pfc_job_setup_mulmods": (u64, [vp, ctypes.c_int]),
            "pfc_job_verify_tables": (ctypes.c_int, [vp, P(u64)]),
            "pfc_finalize_factors": (ctypes.c_int, [ctypes.c_uint, u32, vp, sz, ctypes.c_int,
                                                    ctypes.c_int, P(sz), P(u64)]),
            "pfc_verify_factors_device": (ctypes.c_int, [vp, ctypes.c_uint, u32, vp, sz, vp, P(sz)]),
            "pfc_setup_program_size": (ctypes.c_int, [ctypes.c_uint, u32, ctypes.c_int, P(u64), P(u64)]),
            "pfc_setup_program_eval": (ctypes.c_int, [ctypes.c_uint, u32, ctypes.c_int, u64, P(u64), P(u64)]),
            "pfc_is_prime": (ctypes.c_int, [u64]),
            "pfc_format_factor": (ctypes.c_int, [vp, ctypes.c_char_p, sz]),
            "pfc_status_string": (ctypes.c_char_p, [ctypes.c_int]),
            "pfc_bench_int_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, P(ctypes.c_double)]),
            "pfc_segment_noalloc": (ctypes.c_int, [ctypes.c_uint, u32, u32, u64, u64, vp, u64, vp, vp]),
            "pfc_batch_create": (ctypes.c_int, [vp, P(vp)]),
            "pfc_batch_destroy": (ctypes.c_int, [vp]),
            "pfc_batch_submit": (ctypes.c_int, [vp, P(JobDesc), P(u64)]),
            "pfc_batch_step": (ctypes.c_int, [vp, P(u32), P(u32)]),
            "pfc_batch_result": (ctypes.c_int, [vp, u64, P(BatchStatus)]),
            "pfc_batch_take_hits": (ctypes.c_int, [vp, u64, vp, sz, P(sz)]),
            "pfc_batch_release": (ctypes.c_int, [vp, u64]),
            "pfc_batch_iterations": (u64, [vp]),
            "pfc_batch_set_iteration_work": (ctypes.c_int, [vp, ctypes.c_double]),
            "pfc_batch_set_policy": (ctypes.c_int, [vp, ctypes.c_int]),
            "pfc_batch_set_hit_capacity": (ctypes.c_int, [vp, u32]),
            "pfc_autotune": (ctypes.c_int, [vp, ctypes.c_char_p, sz]),
            "pfc_ctx_set_graphs": (ctypes.c_int, [vp, ctypes.c_int]),
            "pfc_ctx_set_split": (ctypes.c_int, [vp, ctypes.c_int]),
            "pfc_ctx_set_setup_tc": (ctypes.c_int, [vp, ctypes.c_int]),
            "pfc_ctx_set_walk_variant": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
            "pfc_ctx_walk_variant": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, P(ctypes.c_int),
                                                    P(ctypes.c_int), P(ctypes.c_int)]),
            "pfc_batch_timing": (ctypes.c_int, [vp, P(BatchTimes)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(code):
    return lib().pfc_status_string(code).decode()


def _ck(code, where):
    if code != PFC_OK:
        raise PFCError(code, where)


class Context:
    """One GPU, one stream, a device-memory budget (pfc_ctx_create)."""

    def __init__(self, device=0, budget=0):
        self.h = ctypes.c_void_p()
        _ck(lib().pfc_ctx_create(device, budget, ctypes.byref(self.h)), "pfc_ctx_create")
        # the tensor-core setup's state as pfc_ctx_create set it from the environment
        self.setup_tc = os.environ.get("PFCSIEVE_SETUP_TC", "1")[:1] != "0"

    def close(self):
        if self.h:
            lib().pfc_ctx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        """cudaStream_t of the context, as an integer."""
        return lib().pfc_ctx_stream(self.h) or 0

    @property
    def launches(self):
        return lib().pfc_ctx_launch_count(self.h)

    def transfer_bytes(self):
        """(host->device, device->host) bytes copied so far."""
        a, b = ctypes.c_uint64(0), ctypes.c_uint64(0)
        _ck(lib().pfc_ctx_transfer_bytes(self.h, ctypes.byref(a), ctypes.byref(b)), "transfer_bytes")
        return a.value, b.value

    def autotune(self):
        """Time the walk variants on this device and keep the fastest; returns
        the report (one line per variant, * = chosen)."""
        buf = ctypes.create_string_buffer(4096)
        _ck(lib().pfc_autotune(self.h, buf, 4096), "pfc_autotune")
        return buf.value.decode()

    def set_graphs(self, on):
        """Replay each job's segment body as a CUDA graph (default on)."""
        _ck(lib().pfc_ctx_set_graphs(self.h, int(bool(on))), "pfc_ctx_set_graphs")

    def set_split(self, on):
        """Walk small candidate sets in n sub-ranges (default on)."""
        _ck(lib().pfc_ctx_set_split(self.h, int(bool(on))), "pfc_ctx_set_split")

    def set_setup_tc(self, on):
        """Fold the setup's table words on the tensor cores (class 32 and class 64
        below 2^64/3, programs above the word thresholds; default on)."""
        _ck(lib().pfc_ctx_set_setup_tc(self.h, int(bool(on))), "pfc_ctx_set_setup_tc")
        self.setup_tc = bool(on)

    def set_walk_variant(self, cls, fused, variant):
        _ck(lib().pfc_ctx_set_walk_variant(self.h, cls, int(fused), variant), "pfc_ctx_set_walk_variant")

    def walk_variant(self, cls, fused):
        """(variant index, candidates per thread, block length)."""
        v, n, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _ck(lib().pfc_ctx_walk_variant(self.h, cls, int(fused), ctypes.byref(v), ctypes.byref(n),
                                       ctypes.byref(b)), "pfc_ctx_walk_variant")
        return v.value, n.value, b.value

    def device_info(self):
        buf = ctypes.create_string_buffer(256)
        sms = ctypes.c_int(0)
        _ck(lib().pfc_ctx_device_info(self.h, buf, 256, ctypes.byref(sms)), "device_info")
        return buf.value.decode(), sms.value


class Job:
    """One search (mode, [nmin, nmax), [pmin, pmax)); see include/pfcsieve.h."""

    def __init__(self, ctx, mode, nmin, nmax, pmin, pmax):
        self.ctx = ctx
        self.mode, self.nmin, self.nmax, self.pmin, self.pmax = mode, nmin, nmax, pmin, pmax
        self.h = ctypes.c_void_p()
        _ck(lib().pfc_job_create(ctx.h, mode, nmin, nmax, pmin, pmax, ctypes.byref(self.h)),
            "pfc_job_create")

    def close(self):
        if self.h:
            lib().pfc_job_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # stage calls
    def gen(self, lo, hi):
        _ck(lib().pfc_gen_candidates(self.h, lo, hi), "pfc_gen_candidates")

    def setup(self):
        _ck(lib().pfc_setup(self.h), "pfc_setup")

    def iterate(self, lo, hi):
        _ck(lib().pfc_iterate(self.h, lo, hi), "pfc_iterate")

    def check(self):
        _ck(lib().pfc_check(self.h), "pfc_check")

    def segment(self, lo, hi):
        _ck(lib().pfc_segment(self.h, lo, hi), "pfc_segment")

    def segment_end(self, lo):
        hi = ctypes.c_uint64(0)
        _ck(lib().pfc_job_segment_end(self.h, lo, ctypes.byref(hi)), "pfc_job_segment_end")
        return hi.value

    def sync(self):
        _ck(lib().pfc_sync(self.h), "pfc_sync")

    def drain_hits(self):
        n = ctypes.c_size_t(0)
        cap = 1 << 16
        while True:
            buf = np.zeros(cap, dtype=FACTOR_DTYPE)
            rc = lib().pfc_drain_hits(self.h, buf.ctypes.data, cap, ctypes.byref(n))
            if rc == PFC_ERR_HIT_OVERFLOW and n.value > cap:
                cap = n.value
                continue
            _ck(rc, "pfc_drain_hits")
            return buf[: n.value]

    def totals(self):
        t, c = ctypes.c_uint64(0), ctypes.c_uint64(0)
        _ck(lib().pfc_job_totals(self.h, ctypes.byref(t), ctypes.byref(c)), "pfc_job_totals")
        return t.value, c.value

    def run(self, cap=1 << 20):
        """Whole p range; returns the raw hits (unsorted)."""
        while True:
            buf = np.zeros(max(cap, 1), dtype=FACTOR_DTYPE)
            n = ctypes.c_size_t(0)
            rc = lib().pfc_job_run(self.h, buf.ctypes.data, cap, ctypes.byref(n))
            if rc == PFC_ERR_HIT_OVERFLOW:
                raise PFCError(rc, "pfc_job_run: %d hits do not fit %d; rerun with cap=%d"
                               % (n.value, cap, n.value))
            _ck(rc, "pfc_job_run")
            return buf[: n.value]

    def segment_state(self):
        """(p, s0, s1) of the current segment in the reference's R = 2^64 form."""
        n = ctypes.c_size_t(0)
        rc = lib().pfc_segment_state(self.h, None, None, None, 0, ctypes.byref(n))
        if rc not in (PFC_OK, -1):
            _ck(rc, "pfc_segment_state")
        cap = n.value
        p = np.zeros(max(cap, 1), dtype=np.uint64)
        s0 = np.zeros_like(p)
        s1 = np.zeros_like(p)
        _ck(lib().pfc_segment_state(self.h, p.ctypes.data, s0.ctypes.data, s1.ctypes.data, cap,
                                    ctypes.byref(n)), "pfc_segment_state")
        return p[: n.value], s0[: n.value], s1[: n.value]

    @property
    def pairs(self):
        return lib().pfc_job_pairs(self.h)

    def setup_mulmods(self, cls64):
        return lib().pfc_job_setup_mulmods(self.h, int(cls64))

    def verify_tables(self):
        """Device self-check of the job's tables; returns the bytes checked."""
        n = ctypes.c_uint64(0)
        _ck(lib().pfc_job_verify_tables(self.h, ctypes.byref(n)), "pfc_job_verify_tables")
        return n.value


class Batch:
    """Many searches on one device with continuous batching (pfc_batch_*).

    submit() queues a search and returns its id; step() runs one iteration
    (admit queued searches, advance every admitted one, retire finished ones);
    result(id) gives the raw totals and hits of a finished search."""

    def __init__(self, ctx, iteration_work=None, policy=None):
        self.ctx = ctx
        h = ctypes.c_void_p()
        _ck(lib().pfc_batch_create(ctx.h, ctypes.byref(h)), "pfc_batch_create")
        self.h = h
        if iteration_work is not None:
            _ck(lib().pfc_batch_set_iteration_work(self.h, float(iteration_work)),
                "pfc_batch_set_iteration_work")
        if policy is not None:
            _ck(lib().pfc_batch_set_policy(self.h, int(policy)), "pfc_batch_set_policy")

    def close(self):
        if self.h:
            lib().pfc_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, mode, nmin, nmax, pmin, pmax):
        d = JobDesc(mode, nmin, nmax, pmin, pmax)
        i = ctypes.c_uint64(0)
        _ck(lib().pfc_batch_submit(self.h, ctypes.byref(d), ctypes.byref(i)), "pfc_batch_submit")
        return i.value

    def step(self):
        """One iteration; returns (searches running, searches waiting)."""
        a, q = ctypes.c_uint32(0), ctypes.c_uint32(0)
        _ck(lib().pfc_batch_step(self.h, ctypes.byref(a), ctypes.byref(q)), "pfc_batch_step")
        return a.value, q.value

    def status(self, job_id):
        r = BatchStatus()
        _ck(lib().pfc_batch_result(self.h, job_id, ctypes.byref(r)), "pfc_batch_result")
        return r

    def hits(self, job_id):
        n = ctypes.c_size_t(0)
        rc = lib().pfc_batch_take_hits(self.h, job_id, None, 0, ctypes.byref(n))
        if rc not in (PFC_OK, PFC_ERR_HIT_OVERFLOW):
            _ck(rc, "pfc_batch_take_hits")
        buf = np.zeros(max(n.value, 1), dtype=FACTOR_DTYPE)
        _ck(lib().pfc_batch_take_hits(self.h, job_id, buf.ctypes.data, n.value, ctypes.byref(n)),
            "pfc_batch_take_hits")
        return buf[: n.value]

    def release(self, job_id):
        _ck(lib().pfc_batch_release(self.h, job_id), "pfc_batch_release")

    def set_hit_capacity(self, records):
        _ck(lib().pfc_batch_set_hit_capacity(self.h, int(records)), "pfc_batch_set_hit_capacity")

    @property
    def iterations(self):
        return lib().pfc_batch_iterations(self.h)

    def timing(self):
        t = BatchTimes()
        _ck(lib().pfc_batch_timing(self.h, ctypes.byref(t)), "pfc_batch_timing")
        return {k: getattr(t, k) for k, _ in BatchTimes._fields_}

    def run(self):
        """Step until every submitted search has finished."""
        while True:
            a, q = self.step()
            if a == 0 and q == 0:
                return


def verify_factors(ctx, mode, nmax, hits):
    """Re-verify hits on the GPU of `ctx` (pfc_verify_factors_device).

    Returns a bool array, True for each hit whose verification product is not
    the +-1 its sign claims; raises nothing for failing hits."""
    f = np.ascontiguousarray(hits, dtype=FACTOR_DTYPE)
    bad = np.zeros(len(f), dtype=np.uint8)
    failed = ctypes.c_size_t(0)
    rc = lib().pfc_verify_factors_device(ctx.h, mode, nmax, f.ctypes.data if len(f) else None, len(f),
                                         bad.ctypes.data if len(f) else None, ctypes.byref(failed))
    if rc not in (0, -6):
        raise PFCError(rc, "pfc_verify_factors_device")
    return bad.astype(bool)


def finalize(mode, nmax, hits, threads=2, verify=True, ctx=None):
    """Sort, re-verify, drop 2-PRP p and fold n+-1 (cl_sieve.cpp:496-589).

    verify: True re-verifies on the CPU (the reference's check), "device"
    on the GPU of `ctx` (pfc_verify_factors_device), False not at all; a
    failing hit raises PFCError(-6) either way.
    Returns (kept factors sorted by (p, |n|, type), checksum addend)."""
    f = np.ascontiguousarray(hits, dtype=FACTOR_DTYPE).copy()
    if verify == "device":
        if ctx is None:
            raise ValueError("verify='device' needs ctx")
        if verify_factors(ctx, mode, nmax, f).any():
            raise PFCError(-6, "pfc_verify_factors_device")
        verify = False
    kept = ctypes.c_size_t(0)
    add = ctypes.c_uint64(0)
    _ck(lib().pfc_finalize_factors(mode, nmax, f.ctypes.data if len(f) else None, len(f), threads,
                                   int(bool(verify)), ctypes.byref(kept), ctypes.byref(add)),
        "pfc_finalize_factors")
    return f[: kept.value], add.value


def int_peak(device=0, variant=0):
    """Measured integer-pipe throughput in ops/s (see pfc_bench_int_peak)."""
    v = ctypes.c_double(0)
    _ck(lib().pfc_bench_int_peak(device, variant, ctypes.byref(v)), "pfc_bench_int_peak")
    return v.value


def setup_program_size(mode, nmin, wide=True):
    """(table words, squarings) per candidate of a search's setup programs."""
    w, q = ctypes.c_uint64(0), ctypes.c_uint64(0)
    _ck(lib().pfc_setup_program_size(mode, nmin, int(bool(wide)), ctypes.byref(w), ctypes.byref(q)),
        "pfc_setup_program_size")
    return w.value, q.value


SETUP_FORMS = {"narrow": 0, "wide": 1, "paired": 2}


def setup_program_eval(mode, nmin, p, form="wide"):
    """(s0, s1): the starting residues a search's setup programs give for p,
    replayed on the host as the device runs them (pfc_setup_program_eval);
    form "narrow" (64-bit words), "wide" (896-bit words) or "paired" (the
    tensor-core setup's pairs of 896-bit words)."""
    s0, s1 = ctypes.c_uint64(0), ctypes.c_uint64(0)
    _ck(lib().pfc_setup_program_eval(mode, nmin, SETUP_FORMS[form], int(p), ctypes.byref(s0), ctypes.byref(s1)),
        "pfc_setup_program_eval")
    return s0.value, s1.value


def is_prime(p):
    return bool(lib().pfc_is_prime(int(p)))


def format_factor(f):
    a = np.zeros(1, dtype=FACTOR_DTYPE)
    a[0] = f
    buf = ctypes.create_string_buffer(96)
    n = lib().pfc_format_factor(a.ctypes.data, buf, 96)
    if n < 0:
        raise PFCError(n, "pfc_format_factor")
    return buf.value.decode()


@dataclass
class SieveResult:
    factorcount: int
    primecount: int
    checksum: int
    pairs: int
    factors: np.ndarray = field(repr=False)
    hits: int = 0

    def checksum_hex(self):
        return "%016X" % self.checksum


def sieve(mode, nmin, nmax, pmin, pmax, device=0, threads=2, verify=True, ctx=None, segments=4):
    """One complete search, as the reference's cl_sieve() runs it.

    A search of more than about 1e11 pairs (0.1 s of GPU time or more) is
    walked in at least `segments` segments (each at most the size the library
    suggests) and the CPU verification of one segment's hits runs in a worker
    thread while the GPU works on the next (the C calls release the GIL);
    smaller searches run as library-sized segments with one verification at
    the end, where a worker thread and extra segments would cost more than the
    overlap gains.  Segments are disjoint p ranges in increasing order, so the
    concatenated kept factors are sorted and the checksum addends add up: the
    result equals one verification of all hits.  verify="device" checks the
    hits on the GPU (pfc_verify_factors_device) after the last segment instead
    of on the CPU."""
    import concurrent.futures as cf
    import math

    own = ctx is None
    ctx = ctx or Context(device)
    try:
        pairs_est = (pmax - pmin) / math.log(max(pmin, 3)) * max(nmax - nmin, 1)
        parts_wanted = max(segments, 1) if pairs_est >= 1e11 else 1
        on_device = verify == "device"
        cpu_verify = bool(verify) and not on_device
        raw = []   # hits for the device check, which runs on this thread (one thread per context)
        with Job(ctx, mode, nmin, nmax, pmin, pmax) as job:
            if parts_wanted == 1:
                hits = job.run()
                termsum, primecount = job.totals()
                pairs = job.pairs
                raw.append(hits)
                parts = [finalize(mode, nmax, hits, threads=threads, verify=cpu_verify)]
                nhits = len(hits)
            else:
                span = max((pmax - pmin + parts_wanted - 1) // parts_wanted, 1)
                with cf.ThreadPoolExecutor(1) as pool:
                    futs, nhits, lo = [], 0, pmin
                    while lo < pmax:
                        hi = min(job.segment_end(lo), lo + span, pmax)
                        job.segment(lo, hi)
                        h = job.drain_hits()
                        nhits += len(h)
                        raw.append(h)
                        futs.append(pool.submit(finalize, mode, nmax, h, threads, cpu_verify))
                        lo = hi
                    termsum, primecount = job.totals()
                    pairs = job.pairs
                    parts = [f.result() for f in futs]
        if on_device and nhits and verify_factors(ctx, mode, nmax, np.concatenate(raw)).any():
            raise PFCError(-6, "pfc_verify_factors_device")
        kept = np.concatenate([k for k, _ in parts]) if parts else np.zeros(0, dtype=FACTOR_DTYPE)
        add = sum(a for _, a in parts)
        return SieveResult(factorcount=len(kept), primecount=primecount,
                           checksum=(termsum + add) & 0xFFFFFFFFFFFFFFFF, pairs=pairs,
                           factors=kept, hits=nhits)
    finally:
        if own:
            ctx.close()
