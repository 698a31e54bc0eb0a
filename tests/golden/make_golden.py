"""Generate tests/golden/ref_segments.npz from the reference's own kernels.

Run where the reference sources are available (oracle/Makefile `ref` target
compiles kernels/setup.cl, kernels/iterate.cl and verifyprime.cpp for the
CPU into oracle/_ref):

    python tests/golden/make_golden.py

For each small segment below it stores the candidate primes (from the oracle's
restatement of getsegprimes/addsmallprimes), the final per-candidate records
(s4, s6, s7) and the hit list produced by the reference kernels, and for a
sample of integers the reference isPrime() verdicts.  The GPU parity tests
compare the CUDA path with these vectors on machines without the reference.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as o  # noqa: E402

# (mode, nmin, nmax, pmin, pmax): all four modes, both 32- and 64-bit p,
# p <= n (Wilson-type hits), and p near 2^62 / 2^63 / 2^64
SEGMENTS = [
    (1, 101, 3000, 101, 5000),
    (2, 101, 3000, 101, 5000),
    (4, 101, 3000, 101, 5000),
    (5, 101, 3000, 3, 5000),
    (1, 1000, 20000, 10**7, 10**7 + 20000),
    (5, 5000, 9000, 10**9, 10**9 + 20000),
    (2, 2000, 9000, 2**62, 2**62 + 20000),
    (4, 3000, 6000, 2**40, 2**40 + 30000),
    (5, 500, 4000, 2**63 + 1000, 2**63 + 40000),
    (1, 101, 2000, 2**64 - 40000, 2**64 - 1),
    (2, 101, 5000, 2**32 - 30000, 2**32 + 30000),
]


def main():
    if not o.ref_available():
        raise SystemExit("reference kernels not available: cannot regenerate fixtures")
    out = {}
    for i, (mode, nmin, nmax, pmin, pmax) in enumerate(SEGMENTS):
        c = o.candidates(pmin, pmax)
        rec, hits = o.ref_segment(mode, nmin, nmax, c)
        out["seg%d_params" % i] = np.array([mode, nmin, nmax, pmin, pmax], dtype=np.uint64)
        out["seg%d_cands" % i] = c
        out["seg%d_s4s6s7" % i] = rec[:, [4, 6, 7]].copy()
        out["seg%d_hits" % i] = hits
    rng = np.random.default_rng(1)
    sample = np.concatenate([
        np.arange(3, 3000, 2, dtype=np.uint64),
        np.array([42799, 85489, 4294967297, 3215031751, 2152302898747, 3474749660383,
                  341550071728321, 3825123056546413051, 318665857834031151167461 % 2**64],
                 dtype=np.uint64),
        rng.integers(1 << 32, 1 << 63, size=2000, dtype=np.uint64) | np.uint64(1),
    ])
    R = o.ref_lib()
    out["isprime_n"] = sample
    out["isprime_v"] = np.array([R.ref_is_prime(int(x)) for x in sample], dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "ref_segments.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_segments.npz"), "segments:", len(SEGMENTS))


if __name__ == "__main__":
    main()
