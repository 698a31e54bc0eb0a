"""Writes tests/golden/verify_hits_64.npz: true hits with p above 2^32, found
by the oracle's sieve, so that the host re-verification's 64-bit arithmetic
(p >= 2^32) is checked on hits of every type without a GPU.

    python tests/golden/make_verify_hits.py [threads]

Each search is an oracle run over all candidates of its p range (the
oracle's sieve is the reference's algorithm, kernels/setup.cl and
kernels/iterate.cl restated); about a minute on 8 threads.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as o  # noqa: E402

# (mode, nmin, nmax, pmin, pmax): factorial and compositorial hits (-! -c)
# and primorial hits, just above 2^32
SEARCHES = [
    (5, 101, 30000, 2**32, 2**32 + 20_000_000),
    (2, 101, 200000, 2**32 + 20_000_000, 2**32 + 60_000_000),
]


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    out = {}
    for i, (mode, nmin, nmax, pmin, pmax) in enumerate(SEARCHES):
        cands = o.candidates(pmin, pmax)
        hits, _, _ = o.sieve(mode, nmin, nmax, cands, threads)
        hits = o.sort_factors(hits)
        print("search", i, (mode, nmin, nmax, pmin, pmax), len(cands), "candidates", len(hits), "hits")
        out["s%d_params" % i] = np.array([mode, nmin, nmax, pmin, pmax], dtype=np.uint64)
        out["s%d_hits" % i] = hits
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "verify_hits_64.npz"), **out)


if __name__ == "__main__":
    main()
