"""Generate tests/golden/configs.npz: the three single-search benchmark
workloads run in full by the CPU oracle, plus slices of each run through the
reference's own kernels compiled for the CPU (oracle/_ref).

    python tests/golden/make_configs.py            # all three (cfg2 takes ~15 min on 8 cores)
    python tests/golden/make_configs.py cfg1 cfg3  # a subset, merged into the existing file

The workloads are the benchmark searches exactly at their bounds:

    cfg1  -!    -n 101 -N 20000   -p 1e7  -P 1.1e7
    cfg2  -! -c -n 101 -N 200000  -p 1e9  -P 1.1e9
    cfg3  -#    -n 101 -N 1e6     -p 2^62 -P 2^62+5e7

For each the file holds the checksum line value, primecount, factorcount, the
hit count before the 2-PRP filter and the kept factor list sorted by
(p, |n|, type) -- what factors.txt and the checksum line of the reference show
(cl_sieve.cpp:556-589,808-818).  For a slice of candidates at each end of the
p range, the residues and hits of the reference's setup.cl/iterate.cl (built
by `make -C oracle ref`) are stored too and cross-checked against the oracle
before anything is written.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as o  # noqa: E402

OUT = os.path.join(HERE, "configs.npz")

CONFIGS = {
    "cfg1": (o.FACTORIAL, 101, 20000, 10**7, 11 * 10**6),
    "cfg2": (o.FACTORIAL | o.COMPOSITORIAL, 101, 200000, 10**9, 11 * 10**8),
    "cfg3": (o.PRIMORIAL, 101, 10**6, 2**62, 2**62 + 5 * 10**7),
}

SLICE = 1000  # candidates taken from each end of the p range for the reference check


def ref_slices(name, mode, nmin, nmax, pmin, pmax, out):
    cands = o.candidates(pmin, pmax)
    sl = np.concatenate([cands[:SLICE], cands[-SLICE:]])
    rec, rhits = o.ref_segment(mode, nmin, nmax, sl)
    ohits, _, terms = o.sieve(mode, nmin, nmax, sl, want_terms=True)
    rterms = o.ref_terms(mode, rec)
    if not np.array_equal(rterms, terms[:, 3]):
        raise SystemExit("%s: oracle checksum terms differ from the reference kernels" % name)
    if not np.array_equal(rhits, ohits):
        raise SystemExit("%s: oracle hits differ from the reference kernels" % name)
    out[name + "_ref_cands"] = sl
    out[name + "_ref_terms"] = rterms
    out[name + "_ref_hits"] = rhits
    return len(cands)


def main(names):
    out = dict(np.load(OUT)) if os.path.exists(OUT) else {}
    have_ref = o.ref_available()
    for name in names:
        mode, nmin, nmax, pmin, pmax = CONFIGS[name]
        t0 = time.time()
        res, facs = o.job(mode, nmin, nmax, pmin, pmax)
        dt = time.time() - t0
        out[name + "_params"] = np.array([mode, nmin, nmax, pmin, pmax], dtype=np.uint64)
        out[name + "_totals"] = np.array([res.checksum, res.primecount, res.factorcount,
                                          res.hitcount, res.pairs], dtype=np.uint64)
        out[name + "_factors"] = o.sort_factors(facs)
        msg = "%s: %d candidates, %d factors, checksum %016X (%.1f s)" % (
            name, res.primecount, res.factorcount, res.checksum, dt)
        if have_ref:
            ref_slices(name, mode, nmin, nmax, pmin, pmax, out)
            msg += "; reference slice of %d candidates agrees" % (2 * SLICE)
        print(msg, flush=True)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CONFIGS))
