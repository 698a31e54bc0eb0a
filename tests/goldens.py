"""Shared loaders for the committed golden vectors."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def selftest_cases():
    with open(os.path.join(GOLDEN, "selftest_cases.json")) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        c["checksum_int"] = int(c["checksum"], 16)
    return cases


def case(i):
    return [c for c in selftest_cases() if c["id"] == i][0]


def ref_segments():
    d = np.load(os.path.join(GOLDEN, "ref_segments.npz"))
    segs = []
    i = 0
    while "seg%d_params" % i in d:
        mode, nmin, nmax, pmin, pmax = [int(x) for x in d["seg%d_params" % i]]
        segs.append(dict(mode=mode, nmin=nmin, nmax=nmax, pmin=pmin, pmax=pmax,
                         cands=d["seg%d_cands" % i], s4s6s7=d["seg%d_s4s6s7" % i],
                         hits=d["seg%d_hits" % i]))
        i += 1
    return segs, d["isprime_n"], d["isprime_v"]


def terms_from_records(mode, s4s6s7):
    """Checksum term per candidate (kernels/check.cl:59,115,161)."""
    s4, s6, s7 = s4s6s7[:, 0], s4s6s7[:, 1], s4s6s7[:, 2]
    with np.errstate(over="ignore"):
        if mode == 2:
            return s6.copy()
        if mode == 5:
            return s4 + s6 + s7
        return s6 + s7
