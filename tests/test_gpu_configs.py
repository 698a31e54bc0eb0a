"""The three single-search benchmark workloads, run in full on the GPU at their
exact bounds and compared with fixtures the CPU oracle wrote for the same
bounds (tests/golden/configs.npz, made by tests/golden/make_configs.py):

    cfg1  -!    n in [101, 20000)   p in [1e7, 1.1e7)
    cfg2  -! -c n in [101, 200000)  p in [1e9, 1.1e9)
    cfg3  -#    n in [101, 1e6)     p in [2^62, 2^62 + 5e7)

What is compared is what the reference prints: the checksum line, the
candidate count and the kept factor list (factors.txt), bit for bit
(cl_sieve.cpp:556-589,808-818; kernels/check.cl:59,115,161).  A slice of
candidates at each end of every p range is also compared with the output of
the reference's own setup.cl/iterate.cl compiled for the CPU, stored in the
same file.  For cfg1 and cfg2 the factors.txt that the reference's own OpenCL
program wrote on a GB300 (tests/golden/ref_opencl_*_factors.txt, made by
tests/golden/make_ref_opencl.py) is the third pin: the oracle fixture equals
it, and the pfcsieve command line writes the same lines and checksum.
"""
import os

import numpy as np
import pytest

from oracle import oracle as o

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "configs.npz")
NAMES = ["cfg1", "cfg2", "cfg3"]


def fixture(name):
    g = np.load(FIXTURE)
    if name + "_params" not in g:
        pytest.skip("fixture for %s not generated" % name)
    mode, nmin, nmax, pmin, pmax = (int(x) for x in g[name + "_params"])
    checksum, primecount, factorcount, hitcount, pairs = (int(x) for x in g[name + "_totals"])
    return dict(mode=mode, nmin=nmin, nmax=nmax, pmin=pmin, pmax=pmax, checksum=checksum,
                primecount=primecount, factorcount=factorcount, hitcount=hitcount, pairs=pairs,
                factors=g[name + "_factors"],
                ref=(g[name + "_ref_cands"], g[name + "_ref_terms"], g[name + "_ref_hits"])
                if name + "_ref_cands" in g else None)


def test_fixture_bounds_are_the_benchmark_searches():
    want = {"cfg1": (1, 101, 20000, 10**7, 11 * 10**6),
            "cfg2": (5, 101, 200000, 10**9, 11 * 10**8),
            "cfg3": (2, 101, 10**6, 2**62, 2**62 + 5 * 10**7)}
    g = np.load(FIXTURE)
    for name, params in want.items():
        if name + "_params" in g:
            assert tuple(int(x) for x in g[name + "_params"]) == params


def test_cfg1_fixture_reproduced_by_the_oracle():
    """The smallest workload is cheap enough to re-run on the CPU here."""
    f = fixture("cfg1")
    res, facs = o.job(f["mode"], f["nmin"], f["nmax"], f["pmin"], f["pmax"])
    assert (res.checksum, res.primecount, res.factorcount) == (f["checksum"], f["primecount"], f["factorcount"])
    assert np.array_equal(o.sort_factors(facs), f["factors"])


def test_reference_slices_agree_with_the_oracle():
    """The stored reference-kernel outputs equal the oracle on the same
    candidates (at cfg1's size this re-runs in about a second)."""
    f = fixture("cfg1")
    if f["ref"] is None:
        pytest.skip("no reference slice stored")
    cands, terms, hits = f["ref"]
    ohits, _, oterms = o.sieve(f["mode"], f["nmin"], f["nmax"], cands, want_terms=True)
    assert np.array_equal(oterms[:, 3], terms)
    assert np.array_equal(ohits, hits)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_benchmark_search_matches_the_oracle(name):
    import pfcsieve_gb300 as pfc

    f = fixture(name)
    r = pfc.sieve(f["mode"], f["nmin"], f["nmax"], f["pmin"], f["pmax"], threads=os.cpu_count() or 2)
    assert r.primecount == f["primecount"]
    assert r.pairs == f["pairs"]
    assert r.factorcount == f["factorcount"]
    assert np.array_equal(o.sort_factors(r.factors), f["factors"])
    assert "%016X" % r.checksum == "%016X" % f["checksum"]


@pytest.mark.gpu
def test_combined_search_with_device_verification():
    """cfg2 again with the hits checked on the GPU instead of the CPU."""
    import pfcsieve_gb300 as pfc

    f = fixture("cfg2")
    r = pfc.sieve(f["mode"], f["nmin"], f["nmax"], f["pmin"], f["pmax"], verify="device")
    assert (r.checksum, r.primecount, r.factorcount) == (f["checksum"], f["primecount"], f["factorcount"])
    assert np.array_equal(o.sort_factors(r.factors), f["factors"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_reference_slices_on_the_gpu(name):
    """Both ends of each p range against the reference's own kernels: the
    wrapping sum of the checksum terms and the raw hits of the slice."""
    import pfcsieve_gb300 as pfc

    f = fixture(name)
    if f["ref"] is None:
        pytest.skip("no reference slice stored")
    cands, terms, hits = f["ref"]
    half = len(cands) // 2
    with pfc.Context(0) as ctx:
        for sl, lo, hi in [(slice(0, half), f["pmin"], int(cands[half - 1]) + 1),
                           (slice(half, None), int(cands[half]), f["pmax"])]:
            with pfc.Job(ctx, f["mode"], f["nmin"], f["nmax"], lo, hi) as job:
                job.segment(lo, hi)
                termsum, count = job.totals()
                got_hits = o.sort_factors(job.drain_hits())
            assert count == len(cands[sl])
            with np.errstate(over="ignore"):
                want = int(np.sum(terms[sl], dtype=np.uint64))
            assert termsum == want
            sel = (hits["p"] >= lo) & (hits["p"] < hi)
            assert np.array_equal(got_hits, o.sort_factors(hits[sel]))


# ---------------------------------------------- the reference's own OpenCL output

def ref_opencl_file(name):
    path = os.path.join(HERE, "golden", "ref_opencl_%s_factors.txt" % name)
    lines = open(path).read().splitlines()
    body, checksum = lines[:-1], lines[-1]
    if body and body[-1] == "no factors":
        body = body[:-1]
    return body, checksum


def factor_lines(facs):
    """factors.txt lines of factor records (cl_sieve.cpp:565-581)."""
    sym = {0: "!", 1: "#", 2: "!/#"}
    return ["%d | %d%s%+d" % (int(f["p"]), abs(int(f["nc"])), sym[int(f["type"])], -1 if f["nc"] < 0 else 1)
            for f in facs]


@pytest.mark.parametrize("name", ["cfg1", "cfg2"])
def test_reference_opencl_output_equals_the_oracle_fixture(name):
    """The reference's OpenCL program, run on a GB300 at the benchmark
    bounds (tests/golden/make_ref_opencl.py), wrote exactly the oracle's
    factor lines and checksum."""
    f = fixture(name)
    body, checksum = ref_opencl_file(name)
    assert checksum == "%016X" % f["checksum"]
    assert sorted(body) == sorted(factor_lines(f["factors"]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cfg1", "cfg2"])
def test_cli_factors_file_equals_the_reference_opencl_file(name, tmp_path):
    """The drop-in binary on the same search writes the same factors.txt as the
    reference's own program (same lines; the reference writes them in the
    order of its checkpoint drains, here one drain sorted by p as well)."""
    import subprocess

    from pfcsieve_gb300 import build
    build.build()
    cli = os.path.join(os.path.dirname(HERE), "pfcsieve_gb300", "bin", "pfcsieve")
    f = fixture(name)
    flags = {1: ["-!"], 2: ["-#"], 4: ["-c"], 5: ["-!", "-c"]}[f["mode"]]
    args = flags + ["-n", str(f["nmin"]), "-N", str(f["nmax"]), "-p", str(f["pmin"]), "-P", str(f["pmax"]),
                    "-v", str(min(os.cpu_count() or 2, 128))]
    r = subprocess.run([cli] + args, cwd=tmp_path, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    ours = open(tmp_path / "factors.txt").read().splitlines()
    body, checksum = ref_opencl_file(name)
    assert ours[-1] == checksum
    assert sorted(ours[:-1]) == sorted(body)
