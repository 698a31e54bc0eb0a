#!/usr/bin/env python
"""Benchmark of the GB300 sieve path: (p,n) pairs tested per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload combined|factorial|primorial|mixed] [--no-mixed]

Workload (default): the combined factorial + compositorial search (-! -c) over
n in [101, 200000) and p in [10^9, 10^9 + 10^8): about 4.8e6 candidate primes
x 199,899 n = 9.7e11 pairs per step.  Inputs are the scalar search bounds; the
tables live in HBM from job creation on.  The walk kernels are chosen by the
autotuner (pfc_autotune) first; the choice is in config.walk_variants.

One step = candidate generation + setup + iterate over the whole n range +
check + hit read-back, through the C ABI stage calls on the context stream.
`value` is pairs per second over K steps timed with CUDA events on that
stream; the candidate state (16 B x 4.8e6) is smaller than L2, so a 256 MB
buffer is overwritten on the same stream before every step (inside the timed
region).  `e2e` is the same metric through pfcsieve_gb300.sieve(), the call a
user makes: table build and upload, all segments, hit drain, CPU
re-verification of every hit, 2-PRP filter and checksum, timed on the host.

The roofline object covers the iterate (walk) kernel, the dominant one.  The
walk is bound by the integer multiply pipe: each step of a residue chain needs
a fixed set of multiplies (class 32: two 32x32->64 multiplies and one
multiply-low; class 64 below 2^64/3: four 32x32->64 multiplies and one
multiply-low).  Each kind's throughput is measured in
this run (pfc_bench_int_peak); `achieved` is the walk's steps per second x the
IMAD-equivalent cost of a step (each multiply weighted by IMAD rate / its own
rate), `peak` is the IMAD rate, so `frac` is the fraction of time the multiply
pipe would be busy with the algorithm's own multiplies.

Unless --no-mixed, the line also carries `batched`: a sample of the mixed
workload (searches drawn by pfcsieve_gb300.serving.mixed_jobs, seed 0) run as
one batch (pfc_batch_*) and one search at a time (pfc_job_run), with every
search's totals and hits compared between the two, and the same searches
served by the request loop with Poisson arrivals (200 per second, seed 1):
p50 and p99 latency from arrival to result, against the same arrivals served
one at a time.  --workload mixed makes that comparison the headline line.

--impl reference times the reference's CPU path on a bounded sample of the
same workload: its own kernels/setup.cl and kernels/iterate.cl compiled for the
CPU (oracle/_ref/libpfcref.so, OpenMP over all host threads), or the oracle's
restatement of them where the reference sources were not staged.
--impl reference-opencl times the reference's own OpenCL program
(oracle/_ref/pfcsieve_ref, built from its sources) on this GPU end to end, as a
user runs it, with as many verification threads as ours.  The default line
carries the same measurement as `reference_opencl`.  Under torchrun each rank
runs its own p range (weak scaling) and rank 0 prints the JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "(p,n) pairs tested/s"
UNIT = "pairs/s"

WORKLOADS = {
    # configs of the reference benchmark description: -! -c, -!, -#
    "combined": dict(mode=5, nmin=101, nmax=200000, pmin=10**9, pmax=10**9 + 10**8,
                     desc="-! -c n=[101,200000) p=[1e9,1.1e9)"),
    "factorial": dict(mode=1, nmin=101, nmax=20000, pmin=10**7, pmax=10**7 + 10**6,
                      desc="-! n=[101,20000) p=[1e7,1.1e7)"),
    "primorial": dict(mode=2, nmin=101, nmax=10**6, pmin=2**62, pmax=2**62 + 5 * 10**7,
                      desc="-# n=[101,1e6) p=[2^62,2^62+5e7)"),
    # batches of uneven searches (pfcsieve_gb300.serving.mixed_jobs)
    "mixed": dict(mode=0, nmin=0, nmax=0, pmin=0, pmax=0,
                  desc="mixed searches: modes !,#,c; n-range log-uniform [1e3,1e6] from n0 in [101,1e7); "
                       "p-range log-uniform [1e5,1e8] from p0 log-uniform [1e8,2^63]; seed 0"),
    # reduced cases for ncu captures (same kernels)
    "primorial-small": dict(mode=2, nmin=101, nmax=10**6, pmin=2**62, pmax=2**62 + 5 * 10**6,
                            desc="-# n=[101,1e6) p=[2^62,2^62+5e6)"),
    "combined-small": dict(mode=5, nmin=101, nmax=20000, pmin=10**9, pmax=10**9 + 10**7,
                           desc="-! -c n=[101,20000) p=[1e9,1.01e9)"),
    # setup-bound searches of class 64 below 2^64/3 (large n0, short n range)
    # for --setup-ab, and a small one for ncu captures of the setup kernels
    "setup-factorial": dict(mode=1, nmin=9 * 10**6, nmax=9 * 10**6 + 1000, pmin=2**40, pmax=2**40 + 4 * 10**6,
                            desc="-! n=[9e6,9e6+1000) p=[2^40,2^40+4e6)"),
    "setup-combined": dict(mode=5, nmin=5 * 10**6, nmax=5 * 10**6 + 1000, pmin=2**50, pmax=2**50 + 4 * 10**6,
                           desc="-! -c n=[5e6,5e6+1000) p=[2^50,2^50+4e6)"),
    "setup-primorial": dict(mode=2, nmin=9 * 10**6, nmax=9 * 10**6 + 1000, pmin=2**62, pmax=2**62 + 4 * 10**6,
                            desc="-# n=[9e6,9e6+1000) p=[2^62,2^62+4e6)"),
    "setup-factorial32": dict(mode=1, nmin=9 * 10**6, nmax=9 * 10**6 + 1000, pmin=10**9, pmax=10**9 + 4 * 10**6,
                              desc="-! n=[9e6,9e6+1000) p=[1e9,1e9+4e6)"),
    "setup-factorial-small": dict(mode=1, nmin=2 * 10**6, nmax=2 * 10**6 + 100, pmin=2**40, pmax=2**40 + 10**6,
                                  desc="-! n=[2e6,2e6+100) p=[2^40,2^40+1e6)"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "reference-opencl"])
    ap.add_argument("--workload", default="combined", choices=sorted(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="candidates in the CPU baseline sample (0 = auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the batched-vs-plain comparison")
    ap.add_argument("--iteration-work", type=float, default=None,
                    help="batch iteration length in candidate-steps (default: the library's for the policy)")
    ap.add_argument("--mixed-jobs", type=int, default=512,
                    help="searches of the mixed workload (the full set is 512)")
    ap.add_argument("--no-reference-opencl", action="store_true",
                    help="skip timing the reference's OpenCL program")
    ap.add_argument("--setup-ab", action="store_true",
                    help="time the setup kernel of the workload with the integer-pipe and the tensor-core fold")
    ap.add_argument("--capture", action="store_true",
                    help="profiling case: two rounds of the stage calls (gen, setup, iterate, check) on the "
                         "workload with the default walk variants and nothing else, for ncu (-s 1 -c 1 on a "
                         "kernel captures the second round's launch)")
    return ap.parse_args()


# ------------------------------------------------------------ distributed

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    backend = "nccl" if _cuda_available() else "gloo"
    dist.init_process_group(backend=backend)
    return dist


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def shard(wl, rank):
    """Weak scaling: rank r sieves the p range of the same length after rank r-1's."""
    span = wl["pmax"] - wl["pmin"]
    lo = wl["pmin"] + rank * span
    return lo, lo + span


def barrier_max(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if _cuda_available() else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None
        self.thr = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thr = threading.Thread(target=self._read, daemon=True)
        self.thr.start()

    def _read(self):
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 7:
                self.rows.append(f)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thr is not None:
            self.thr.join(timeout=2)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, mx, reasons = [], [], set()
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if r[3 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            # a timed region shorter than the first sample: one reading taken
            # right after it, marked as such
            out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
                   "note": "timed region shorter than the 200 ms sampling interval"}
            try:
                r = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                    "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                   timeout=10).stdout.strip().split(",")
                f = [x.strip() for x in r]
                out["after_region"] = {"sm_mhz": float(f[0]), "sm_max_mhz": float(f[1]),
                                       "reasons": [n for k, n in enumerate(names)
                                                   if f[3 + k].lower().startswith("active")]}
            except Exception:
                pass
            return out
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------- CPU baseline (oracle)

def cpu_kind():
    """'reference' when the reference's own kernels are built for the CPU
    (oracle/_ref/libpfcref.so), else 'port' (the oracle's restatement)."""
    from oracle import oracle as o
    o.build()
    return "reference" if o.ref_available() else "port"


REF_HIT_CAP = 1 << 24


def ref_nstep(ncand):
    """n per iterate launch of the reference kernels on the CPU: the kernels
    append hits without a bound, so a launch may cover at most
    REF_HIT_CAP / (2 x candidates) n (two hits per candidate and n at most)."""
    return int(max(1, min(20000, REF_HIT_CAP // (2 * max(ncand, 1)))))


def cpu_sample_run(wl, ncands, offset=0, kind="port"):
    """Time the reference's CPU path on `ncands` candidates of the workload's
    p range with all host threads: kind 'reference' runs the reference's own
    setup/iterate kernels compiled for the CPU, 'port' the oracle."""
    from oracle import oracle as o
    o.build()
    # candidates of a short range at the bottom of the workload's p range
    lo = wl["pmin"] + offset
    span = max(int(ncands * np.log(float(lo)) * 1.3), 1000)
    cands = o.candidates(lo, lo + span)[:ncands]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    if kind == "reference":
        # iterate chunks sized so that the kernels' unbounded hit appends fit
        o.ref_segment(wl["mode"], wl["nmin"], wl["nmax"], cands, nstep=ref_nstep(len(cands)), hit_cap=REF_HIT_CAP)
    else:
        o.sieve(wl["mode"], wl["nmin"], wl["nmax"], cands, threads)
    dt = time.perf_counter() - t0
    pairs = len(cands) * (wl["nmax"] - wl["nmin"])
    return pairs / dt, dict(cores=threads, seconds=dt, cands=len(cands), pairs=pairs)


CPU_KIND_TEXT = {"reference": "the reference's kernels/setup.cl + kernels/iterate.cl compiled for the CPU "
                              "(oracle/_ref/libpfcref.so), OpenMP over candidates",
                 "port": "the oracle's restatement of the reference kernels (oracle/liboracle.so), "
                         "OpenMP over candidates"}


# ------------------------------------------------- reference OpenCL program

MODE_FLAGS = {1: ["-!"], 2: ["-#"], 4: ["-c"], 5: ["-!", "-c"]}


def _ref_opencl_run(exe, wl, lo, hi, threads, timeout):
    import re
    import tempfile
    cmd = [exe] + MODE_FLAGS[wl["mode"]] + ["-n", str(wl["nmin"]), "-N", str(wl["nmax"]),
                                            "-p", str(lo), "-P", str(hi), "-v", str(threads)]
    with tempfile.TemporaryDirectory() as d:
        t = time.perf_counter()
        r = subprocess.run(cmd, cwd=d, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                           timeout=timeout)
        wall = time.perf_counter() - t
    m = re.search(r"factors (\d+), prime count (\d+), checksum ([0-9A-F]{16})", r.stdout)
    if r.returncode != 0 or not m:
        tail = (r.stdout + r.stderr).strip().splitlines()[-1:] or ["no output"]
        raise RuntimeError("reference OpenCL program failed (rc %d): %s" % (r.returncode, tail[0]))
    return wall, int(m.group(1)), int(m.group(2)), m.group(3)


def reference_opencl(wl, lo, hi, runs=1):
    """The reference's OpenCL program (built from its sources with the
    standalone BOINC and prime-list stand-ins, oracle/Makefile `refcl`) run on
    this GPU over the same search, timed from process start to exit: JIT
    build of its kernels (cached by the driver after the first run), tables,
    sieve, CPU verification of every factor, factors.txt.  A run over a
    1,000-wide p range at the bottom of the range first warms the kernel cache
    and measures the fixed costs; `sieve_pairs_per_s` takes them out."""
    exe = os.path.join(ROOT, "oracle", "_ref", "pfcsieve_ref")
    chk = os.path.join(ROOT, "oracle", "_ref", "refcl_check")
    if not (os.path.exists(exe) and os.path.exists(chk)):
        return {"unavailable": "reference OpenCL program not built (reference sources not staged)"}
    r = subprocess.run([chk], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    if r.returncode != 0:
        return {"unavailable": "OpenCL dispatch check failed: %s" % (r.stdout.strip().splitlines()[-1:] or [""])[0]}
    threads = os.cpu_count() or 1
    try:
        fixed, _, _, _ = _ref_opencl_run(exe, wl, lo, lo + 1000, threads, 600)
        walls, res = [], None
        for _ in range(max(1, runs)):
            w, fc, pc, ck = _ref_opencl_run(exe, wl, lo, hi, threads, 3600)
            walls.append(w)
            res = (fc, pc, ck)
    except Exception as e:   # noqa: BLE001
        return {"unavailable": str(e)}
    wall = float(np.mean(walls))
    pairs = res[1] * (wl["nmax"] - wl["nmin"])
    return {"program": "oracle/_ref/pfcsieve_ref (the reference's main.cpp, cl_sieve.cpp, simpleCL.c, "
                       "kernels/*.cl; OpenCL on this GPU)",
            "wall_s": wall, "runs": len(walls), "fixed_s": fixed, "verify_threads": threads,
            "e2e_pairs_per_s": pairs / wall,
            "sieve_pairs_per_s": pairs / max(wall - fixed, 1e-9),
            "pairs": int(pairs), "factors": res[0], "primecount": res[1], "checksum": res[2]}


def auto_sample(wl):
    # about 10-20 s of CPU work on 16 cores at ~1e8 mulmods/s/core
    per_cand = (wl["nmax"] - wl["nmin"]) * (2 if wl["mode"] == 5 else 1)
    if wl["mode"] == 2:
        per_cand = (wl["nmax"] - wl["nmin"]) / 12 * 2 * 5   # primes only, 64-bit, 2 mulmods
    budget = 1.6e9 * 12 * (os.cpu_count() or 1) / 16
    return int(max(64, min(200000, budget / per_cand)))


# -------------------------------------------------------------- reference

def run_reference(args, wl, world, rank):
    if rank != 0:
        return
    kind = cpu_kind()
    n = args.cpu_sample or max(16, auto_sample(wl) // 4)
    pairs, secs = 0, 0.0
    info = None
    for s in range(args.warmup + args.steps):
        rate, info = cpu_sample_run(wl, n, offset=s * 1000, kind=kind)
        if s >= args.warmup:
            pairs += info["pairs"]
            secs += info["seconds"]
    value = pairs / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (deterministic search bounds)",
        "config": {"workload": wl["desc"], "sample": "%d candidates x full n range per step" % n,
                   "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["cores"], "kind": kind,
                         "sample": "%d candidates from the bottom of the p range x all n; %s"
                                   % (n, CPU_KIND_TEXT[kind])},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_opencl_line(args, wl, rank):
    """--impl reference-opencl: the reference's OpenCL program on this GPU."""
    if rank != 0:
        return
    lo, hi = shard(wl, 0)
    r = reference_opencl(wl, lo, hi, runs=args.steps)
    if "unavailable" in r:
        print(json.dumps({"impl": "reference-opencl", "unavailable": r["unavailable"]}), flush=True)
        return
    line = {
        "impl": "reference-opencl", "metric": METRIC, "value": r["e2e_pairs_per_s"], "unit": UNIT,
        "n_gpus": 1, "steps": r["runs"], "warmup": 1, "ms_per_step": r["wall_s"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (deterministic search bounds)",
        "config": {"workload": wl["desc"], "l2": "n/a (whole program per step)"},
        "e2e": {"value": r["e2e_pairs_per_s"], "unit": UNIT, "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": None},
        "reference_opencl": r,
    }
    print(json.dumps(line), flush=True)


def run_reference_mixed(args, rank):
    """The reference algorithm's CPU form on the mixed workload: each step
    sieves a sample of one search's candidates (bottom of its p range) over
    its whole n range, setup included, searches taken in order."""
    if rank != 0:
        return
    from oracle import oracle as o
    from pfcsieve_gb300 import serving as sv
    kind = cpu_kind()
    jobs = sv.mixed_jobs(512, seed=0)
    threads = os.cpu_count() or 1
    pairs_t, secs_t, samples = 0, 0.0, []
    for step in range(args.warmup + args.steps):
        s = jobs[step % len(jobs)]
        n0 = max(s.nmin, 3)
        setup = n0 / np.log(n0) * 1.3 if s.mode != 2 else n0 / np.log(n0) / 2
        per_cand = setup + (s.nmax - s.nmin)
        m = int(max(16, min(20000, 3e9 * threads / 16 / per_cand)))
        span = max(int(m * np.log(float(s.pmin)) * 1.3), 1000)
        cands = o.candidates(s.pmin, min(s.pmin + span, s.pmax))[:m]
        t = time.perf_counter()
        if kind == "reference":
            o.ref_segment(s.mode, s.nmin, s.nmax, cands, nstep=ref_nstep(len(cands)), hit_cap=REF_HIT_CAP)
        else:
            o.sieve(s.mode, s.nmin, s.nmax, cands, threads)
        dt = time.perf_counter() - t
        if step >= args.warmup:
            pairs_t += len(cands) * (s.nmax - s.nmin)
            secs_t += dt
            samples.append(len(cands))
    value = pairs_t / secs_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs_t / max(args.steps, 1) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded search bounds)",
        "config": {"workload": WORKLOADS["mixed"]["desc"],
                   "sample": "per step one search of the set (in order): %s candidates x its full n range, "
                             "setup included" % samples, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": "candidates %s of searches %d.. of the mixed set; %s"
                                   % (samples, args.warmup, CPU_KIND_TEXT[kind])},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------------- ours

def n_composites(nmin, nmax):
    sieve = np.ones(nmax, dtype=bool)
    sieve[:2] = False
    for i in range(2, int(nmax ** 0.5) + 1):
        if sieve[i]:
            sieve[i * i::i] = False
    seg = sieve[nmin:nmax]
    return int(len(seg) - seg.sum()), int(seg.sum())


def step_recipe(cls32, lazy):
    """Multiplies of one walk step (see arith.cuh): redc31s, redc64l, redc64_u32."""
    if cls32:
        return {"imad_wide": 2, "imad": 1}
    if lazy:
        return {"imad_wide": 4, "imad": 1}
    return {"imad_wide": 7, "imad": 2}


def hit_order(f):
    """Hits sorted by (p, |n|, type, nc), for comparing two runs."""
    if len(f) == 0:
        return f
    return f[np.lexsort((f["nc"], f["type"], np.abs(f["nc"].astype(np.int64)), f["p"]))]


# programs below these sizes (896-bit words, both programs of a search) keep the
# integer-pipe setup when the tensor-core setup is on: kTcMinWords32 and
# kTcMinWords64 of pfcsieve_gb300/csrc/kernels.cuh
TC_MIN_WORDS = {32: 448, 64: 480}


def mixed_roofline(jobs, outcomes, seconds, peaks, tc_s=0.0, setup_tc=True):
    """Multiply-pipe roofline of a batched run: the algorithmic multiplies of
    every search (per candidate: its setup program's table words and squarings
    -- pfc_setup_program_size -- and its walk steps: n for !, composite n for
    the compositorial, prime n for #, both for -! -c), weighted by the measured
    issue rates (IMAD 1, IMAD.WIDE and IMAD.HI by their rates relative to
    IMAD), over the batch's wall time inside pfc_batch_step (iterations and
    the tensor-core setups of admitted searches overlap).  Per unit (see
    arith.cuh, walk.cuh, setup_tc.cu): 896-bit word on the integer pipe
    36 IMAD.WIDE + 2 IMAD (class 32), 76 + 3 (class 64 below 2^64/3); with the
    tensor-core setup, which multiplies pairs of them into 1792-bit words, per
    896-bit word 1.5 + 1 (class 32: half a 32-bit reduction and half a
    Montgomery product) and 5 + 1.5 (class 64: half the one-round reduction and
    half the two-round product), with the fold's 112 x 4 (class 32) or 112 x 8
    (class 64) byte-plane multiply-adds per 896-bit word on the tensor pipe,
    reported apart against the measured dense bf16 peak (fp16 runs at the same
    rate), for programs of at least TC_MIN_WORDS words (smaller ones keep the
    integer-pipe setup); 64-bit
    word and class-64 squaring 8 IMAD.WIDE + 2 IMAD; class-32 squaring
    IMAD.WIDE + IMAD + IMAD.HI; walk steps as step_recipe.  Restores,
    corrections and replays are overhead, as in the single-search roofline.
    A search whose p range crosses 2^31 or 2^64/3 is counted in the class of
    its upper end."""
    import pfcsieve_gb300 as pfc
    w = peaks["imad"] / peaks["imad_wide"]
    h = peaks["imad"] / peaks["mul_hi"]
    lazy_end = 0x5555555555555556
    unit = {32: (36 * w + 2, w + 1 + h), 64: (76 * w + 3, 8 * w + 2), 65: (8 * w + 2, 8 * w + 2)}
    tc_word = {32: 1.5 * w + 1, 64: 5 * w + 1.5}
    tc_macs = 0.0
    top = max(s.nmax for s in jobs) + 1
    isp = np.ones(top, dtype=bool)
    isp[:2] = False
    for i in range(2, int(top ** 0.5) + 1):
        if isp[i]:
            isp[i * i::i] = False
    pc = np.concatenate([[0], np.cumsum(isp)])   # pc[n] = primes below n
    total, crossing, sizes = 0.0, 0, {}
    for i, s in enumerate(jobs):
        cls = 32 if s.pmax <= 2**31 else (64 if s.pmax <= lazy_end else 65)
        crossing += int(s.pmin < 2**31 < s.pmax or s.pmin < lazy_end < s.pmax)
        key = (s.mode, s.nmin, cls != 65)
        if key not in sizes:
            sizes[key] = pfc.setup_program_size(*key)
        words, sq = sizes[key]
        n = s.nmax - s.nmin
        primes = int(pc[s.nmax] - pc[s.nmin])
        steps = {1: n, 2: primes, 4: n - primes, 5: 2 * n - primes}[s.mode]
        recipe = step_recipe(cls == 32, cls == 64)
        step = sum(k * peaks["imad"] / peaks[name] for name, k in recipe.items())
        cw, cs = unit[cls]
        tc = setup_tc and cls in (32, 64) and words >= TC_MIN_WORDS[cls]
        if tc:
            cw = tc_word[cls]
            tc_macs += outcomes[i].primecount * words * 112 * (8 if cls == 64 else 4)
        total += outcomes[i].primecount * (words * cw + sq * cs + steps * step)
    achieved = total / seconds
    return {"bound": "int (multiply pipe)", "achieved": achieved / 1e12, "peak": peaks["imad"] / 1e12,
            "unit": "Tops/s IMAD-equivalent (IMAD.WIDE, IMAD.HI weighted by measured rates)",
            "frac": achieved / peaks["imad"], "traffic": None,
            "kernel": "batch_kernel and setup_tc_kernel (every class and kind of the batch, over its wall time)",
            "alg_ops": total, "seconds": seconds, "searches_crossing_a_class_boundary": crossing,
            "peak_source": "measured in this run (pfc_bench_int_peak, 32-bit IMAD chains)",
            "tensor_setup": tensor_line(2 * tc_macs, seconds)}


def tensor_line(flops, seconds):
    """The tensor-core setups' fold over the batch's wall time (the setups
    overlap the iterations), against the measured dense bf16 peak
    (MEASURED_PEAKS.json, burst)."""
    if not flops or not seconds:
        return None
    peak = None
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except (OSError, ValueError, KeyError):
        pass
    achieved = flops / seconds / 1e12
    return {"flops": flops, "seconds": seconds, "achieved_tflops": achieved, "peak_tflops": peak,
            "frac": achieved / peak if peak else None,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if peak else None}


def run_mixed(ctx, njobs, warmup, steps=1, iteration_work=None, peaks=None):
    """Mixed-workload sample: one batch vs one search at a time, results
    compared search by search, then the request loop under Poisson arrivals."""
    import pfcsieve_gb300 as pfc
    from pfcsieve_gb300 import serving as sv

    jobs = sv.mixed_jobs(512, seed=0)[:njobs]
    sv.run_batched(ctx, jobs[:4], keep_hits=False)       # warm-up: kernels loaded, pools grown
    runs = []
    for _ in range(max(1, steps)):
        runs.append(sv.run_batched(ctx, jobs, iteration_work=iteration_work))
    out_b, t_b, timing = min(runs, key=lambda r: r[1])
    out_p, t_p, service, create = sv.run_plain(ctx, jobs)
    same = all((out_b[i].term_checksum, out_b[i].primecount) == (out_p[i].term_checksum, out_p[i].primecount)
               and np.array_equal(hit_order(out_b[i].hits), hit_order(out_p[i].hits))
               for i in range(len(jobs)))
    # the user's result of every search: verified factors and checksum (hits
    # re-verified on the GPU, sorted and filtered on the CPU)
    t = time.perf_counter()
    for i, s in enumerate(jobs):
        pfc.finalize(s.mode, s.nmax, out_b[i].hits, threads=os.cpu_count() or 1, verify="device", ctx=ctx)
    t_fin = time.perf_counter() - t
    pairs = sum(out_b[i].primecount * (s.nmax - s.nmin) for i, s in enumerate(jobs))
    arrivals = sv.poisson_arrivals(len(jobs), 200.0, seed=1)
    out_s, lat, makespan = sv.serve(ctx, jobs, arrivals)
    same_s = all((out_s[i].term_checksum, out_s[i].primecount) == (out_p[i].term_checksum, out_p[i].primecount)
                 for i in range(len(jobs)))
    lat_p = sv.fcfs_latencies(arrivals, service)
    roof = mixed_roofline(jobs, out_b, timing["step_s"], peaks, tc_s=timing["setup_tc_s"],
                          setup_tc=ctx.setup_tc) if peaks else None
    return {
        "workload": "first %d of the 512 mixed searches (seed 0)" % len(jobs),
        "pairs": int(pairs),
        "batched_pairs_per_s": pairs / t_b,
        "batched_gpu_pairs_per_s": pairs / timing["gpu_s"],
        "plain_pairs_per_s": pairs / t_p,
        "batched_over_plain": t_p / t_b,
        "batched_s": t_b, "plain_s": t_p, "plain_table_build_s": create, "finalize_s": t_fin,
        "finalize_verify": "device",
        "iterations": int(timing["iterations"]), "tasks": int(timing["tasks"]),
        "batched_time": {k: timing[k] for k in ("gpu_s", "setup_tc_s", "prep_s", "admit_s", "step_s")},
        "iteration_work": iteration_work if iteration_work else "default (1.6e12 candidate-steps, throughput policy)",
        "identical_results": bool(same and same_s),
        "roofline": roof,
        "serving": {"arrivals_per_s": 200.0, "makespan_s": makespan,
                    "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                    "plain_fcfs_p50_s": float(np.percentile(lat_p, 50)),
                    "plain_fcfs_p99_s": float(np.percentile(lat_p, 99)),
                    # offered load: arrival rate x mean one-at-a-time service time
                    "rho": 200.0 * float(np.mean(service)),
                    "throughput_pairs_per_s": pairs / makespan},
    }


def run_mixed_line(args, local):
    """--workload mixed: the batched-vs-plain comparison as the headline."""
    import pfcsieve_gb300 as pfc
    ctx = pfc.Context(local, budget=120 * 10**9)
    name, sms = ctx.device_info()
    launches0 = ctx.launches
    h2d0, d2h0 = ctx.transfer_bytes()
    clk = ClockSampler(local)
    clk.start()
    peaks = {k: pfc.int_peak(local, v) for k, v in
             (("imad", 0), ("mul_hi", 1), ("imad_wide", 2), ("iadd_xor", 3))}
    r = run_mixed(ctx, args.mixed_jobs, args.warmup, steps=args.steps, iteration_work=args.iteration_work,
                  peaks=peaks)
    clocks = clk.stop()
    h2d1, d2h1 = ctx.transfer_bytes()
    launches = ctx.launches - launches0
    ctx.close()
    steps = args.steps + 2   # batched runs, the plain run, the served run
    line = {
        "metric": METRIC, "value": r["batched_pairs_per_s"], "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": 1, "ms_per_step": r["batched_s"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32/u64",
        "data": "synthetic (seeded search bounds)",
        "config": {"workload": WORKLOADS["mixed"]["desc"], "searches": args.mixed_jobs,
                   "l2": "per-search state streams through L2; tables re-read per task",
                   "parallelism": "1 GPU, batched", "device": name, "sms": sms},
        "e2e": {"value": r["pairs"] / (r["batched_s"] + r["finalize_s"]), "unit": UNIT,
                "h2d_bytes_per_step": (h2d1 - h2d0) // steps, "d2h_bytes_per_step": (d2h1 - d2h0) // steps},
        "gpu_launches": int(launches), "clocks": clocks, "batched": r,
        "roofline": r["roofline"], "cpu_baseline": None,
    }
    print(json.dumps(line), flush=True)


def run_ours(args, wl, world, rank, local, dist):
    import torch

    import pfcsieve_gb300 as pfc

    torch.cuda.set_device(local)
    lo, hi = shard(wl, rank)
    ctx = pfc.Context(local)
    name, sms = ctx.device_info()
    ctx.autotune()
    tuned = {"%s/%s" % (c, "fused" if f else "single"): "nc=%d b=%d" % ctx.walk_variant(i, f)[1:]
             for i, c in ((0, "class32"), (1, "class64-lazy")) for f in (0, 1)}
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    job = pfc.Job(ctx, wl["mode"], wl["nmin"], wl["nmax"], lo, hi)

    ncomp, nprime = n_composites(wl["nmin"], wl["nmax"])
    it_ms = []

    def step():
        with torch.cuda.stream(stream):
            flush.zero_()
        job.gen(lo, hi)
        job.setup()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        job.iterate(wl["nmin"], wl["nmax"])
        b.record(stream)
        job.check()
        job.drain_hits()
        return a, b

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(dist)
    launches0 = ctx.launches
    pairs0 = job.pairs
    clk = ClockSampler(local)
    clk.start()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    evs = [step() for _ in range(args.steps)]
    t1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    barrier(dist)
    ms = t0.elapsed_time(t1)
    it_ms = [a.elapsed_time(b) for a, b in evs]
    launches = ctx.launches - launches0
    pairs = job.pairs - pairs0
    ms_max = barrier_max(dist, ms)
    pairs_total = pairs * world
    value = pairs_total / (ms_max * 1e-3)

    termsum, _ = job.totals()
    setup_mm = int(job.setup_mulmods(0 if hi <= 2**31 else 1))
    cands_per_step = pairs // args.steps // (wl["nmax"] - wl["nmin"])
    job.close()

    # roofline of the iterate kernel: algorithmic 32-bit multiply ops / time
    mode = wl["mode"]
    if mode == 2:
        steps_per_cand = nprime
    elif mode == 5:
        steps_per_cand = (wl["nmax"] - wl["nmin"]) + ncomp
    elif mode == 4:
        steps_per_cand = ncomp
    else:
        steps_per_cand = wl["nmax"] - wl["nmin"]
    cls32 = hi <= 2**31
    lazy = hi <= 0x5555555555555556
    peaks = {k: pfc.int_peak(local, v) for k, v in
             (("imad", 0), ("mul_hi", 1), ("imad_wide", 2), ("iadd_xor", 3))}
    recipe = step_recipe(cls32, lazy)
    imad_eq = sum(n * peaks["imad"] / peaks[k] for k, n in recipe.items())
    walk_steps = cands_per_step * steps_per_cand
    it_s = float(np.mean(it_ms)) * 1e-3
    peak = peaks["imad"]
    achieved = walk_steps * imad_eq / it_s
    alg_ops = walk_steps * imad_eq
    # DRAM bytes of the walk launches of one step, from the committed ncu
    # capture of this workload (profiles/walk_kernel_traffic.json)
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "walk_kernel_traffic.json")
    if os.path.exists(tfile):
        try:
            t = json.load(open(tfile))
            if t.get("workload") == wl["desc"]:
                traffic = t.get("dram_bytes_per_step")
        except Exception:
            traffic = None

    # end to end through the public call
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        h2d0, d2h0 = ctx.transfer_bytes()
        walls = []
        res = None
        for _ in range(args.e2e_steps):
            t = time.perf_counter()
            res = pfc.sieve(mode, wl["nmin"], wl["nmax"], lo, hi, threads=os.cpu_count() or 1,
                            ctx=ctx)
            walls.append(time.perf_counter() - t)
        h2d1, d2h1 = ctx.transfer_bytes()
        e2e = {"value": res.pairs / float(np.mean(walls)), "unit": UNIT,
               "h2d_bytes_per_step": (h2d1 - h2d0) // args.e2e_steps,
               "d2h_bytes_per_step": (d2h1 - d2h0) // args.e2e_steps,
               "seconds_per_step": float(np.mean(walls)),
               "factors": int(res.factorcount), "checksum": res.checksum_hex()}

    ctx.close()

    batched = None
    if rank == 0 and not args.no_mixed:
        # the mixed workload's own context, under the 120 GB device budget of
        # the serving configuration
        mctx = pfc.Context(local, budget=120 * 10**9)
        batched = run_mixed(mctx, args.mixed_jobs, args.warmup, iteration_work=args.iteration_work, peaks=peaks)
        batched["budget_bytes"] = 120 * 10**9
        mctx.close()

    ref_cl = None
    if rank == 0 and not args.no_reference_opencl:
        ref_cl = reference_opencl(wl, lo, hi)
        if e2e is not None and "checksum" in ref_cl:
            ref_cl["same_checksum_and_factor_count"] = (ref_cl["checksum"] == e2e["checksum"]
                                                        and ref_cl["factors"] == e2e["factors"])
            ref_cl["our_e2e_over_reference_e2e"] = e2e["value"] / ref_cl["e2e_pairs_per_s"]

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        kind = cpu_kind()
        n = args.cpu_sample or auto_sample(wl)
        rate, info = cpu_sample_run(wl, n, kind=kind)
        cpu = {"value": rate, "unit": UNIT, "cores": info["cores"], "kind": kind,
               "sample": "%d candidates from the bottom of the p range x all %d n (%.1f s); %s"
                         % (info["cands"], wl["nmax"] - wl["nmin"], info["seconds"], CPU_KIND_TEXT[kind])}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32" if cls32 else "u64",
            "data": "synthetic (deterministic search bounds, as the reference's CLI takes them)",
            "config": {"workload": wl["desc"], "candidates_per_gpu": int(cands_per_step),
                       "pairs_per_step": int(pairs_total // args.steps),
                       "l2": "256 MB buffer overwritten before each step (candidate state < L2)",
                       "parallelism": "p-range shards, one per GPU" if world > 1 else "1 GPU",
                       "device": name, "sms": sms, "walk_variants": tuned},
            "roofline": {"bound": "int (multiply pipe)", "achieved": achieved / 1e12, "peak": peak / 1e12,
                         "unit": "Tops/s IMAD-equivalent (IMAD.WIDE, IMAD.HI weighted by measured rates)",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "walk_kernel<%s>" % ("Cls32" if cls32 else ("Cls64L" if lazy else "Cls64")),
                         "walk_steps_per_step": int(walk_steps),
                         "multiplies_per_walk_step": recipe,
                         "imad_equivalent_per_walk_step": imad_eq,
                         "alg_ops_per_step": alg_ops,
                         "kernel_ms_per_step": it_s * 1e3,
                         "peak_source": "measured in this run (pfc_bench_int_peak, 32-bit IMAD chains)",
                         "int_peaks_tops": {k: v / 1e12 for k, v in peaks.items()},
                         # not a roofline fraction: the same steps priced at the
                         # reference's 20 IMAD-class operations per 64-bit Montgomery
                         # multiplication, over the peak (above 1 where this path's
                         # 32-bit steps do that work in less multiply-pipe time)
                         "reference_cost_model_ratio": walk_steps / it_s * 20 / peak},
            "mulmods": {"walk_per_s": walk_steps * args.steps / (ms_max * 1e-3) * world,
                        "walk_per_pair": steps_per_cand / (wl["nmax"] - wl["nmin"]),
                        "setup_per_candidate": setup_mm},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks,
            "checksum_terms": "%016X" % termsum,
        }
        if batched is not None:
            line["batched"] = batched
        if ref_cl is not None:
            line["reference_opencl"] = ref_cl
        print(json.dumps(line), flush=True)


def run_setup_ab(wl, reps=3):
    """The workload's setup kernel with the table-word fold on the integer
    pipe and on the tensor cores (pfc_ctx_set_setup_tc): the median of `reps`
    CUDA-event timings of pfc_setup on the context stream after the same
    candidate generation, then the whole search, whose totals must agree."""
    import torch

    import pfcsieve_gb300 as pfc
    line = {"setup_ab": wl["desc"]}
    totals = {}
    for tc in (False, True):
        with pfc.Context(0) as ctx:
            ctx.set_setup_tc(tc)
            stream = torch.cuda.ExternalStream(ctx.stream)
            with pfc.Job(ctx, wl["mode"], wl["nmin"], wl["nmax"], wl["pmin"], wl["pmax"]) as job:
                ms = []
                for _ in range(reps + 1):
                    job.gen(wl["pmin"], wl["pmax"])
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    job.setup()
                    b.record(stream)
                    job.iterate(wl["nmin"], wl["nmax"])
                    job.check()
                    job.drain_hits()
                    torch.cuda.synchronize()
                    ms.append(a.elapsed_time(b))
                termsum, count = job.totals()
        key = "tensor" if tc else "integer"
        line[key + "_setup_ms"] = float(np.median(ms[1:]))
        totals[key] = (termsum, count)
    line["candidates"] = totals["tensor"][1] // (reps + 1)
    line["identical_totals"] = totals["tensor"] == totals["integer"]
    line["speedup"] = line["integer_setup_ms"] / line["tensor_setup_ms"]
    print(json.dumps(line), flush=True)


def run_capture(wl):
    """Two rounds of the stage calls on a fresh context, for profilers."""
    import pfcsieve_gb300 as pfc
    with pfc.Context(0) as ctx, pfc.Job(ctx, wl["mode"], wl["nmin"], wl["nmax"], wl["pmin"], wl["pmax"]) as job:
        for _ in range(2):
            job.gen(wl["pmin"], wl["pmax"])
            job.setup()
            job.iterate(wl["nmin"], wl["nmax"])
            job.check()
            job.drain_hits()
        termsum, count = job.totals()
    print(json.dumps({"capture": wl["desc"], "candidates": count // 2, "checksum_terms": "%016X" % termsum}))


def main():
    args = parse()
    wl = WORKLOADS[args.workload]
    if args.capture:
        run_capture(wl)
        return
    if args.setup_ab:
        run_setup_ab(wl)
        return
    world, rank, local = dist_env()
    dist = dist_init(world)
    if args.impl == "reference-opencl":
        run_reference_opencl_line(args, wl, rank)
    elif args.impl == "reference":
        if args.workload == "mixed":
            run_reference_mixed(args, rank)
        else:
            run_reference(args, wl, world, rank)
    elif args.workload == "mixed":
        if rank == 0:
            run_mixed_line(args, local)
    else:
        run_ours(args, wl, world, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
