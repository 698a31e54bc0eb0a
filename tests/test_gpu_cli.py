"""The pfcsieve command line end to end on the GPU: the drop-in surface.

* factors.txt of a reference self-test range holds the oracle's factor lines
  (as a multiset) and the reference's checksum line;
* `pfcsieve -s` runs the reference's 16 self-test ranges and passes them all;
* a run that dies after a checkpoint (a host-side exit injected between
  segments) and is started again resumes from stateA/B.ckp and ends with the
  same factor lines and checksum as an uninterrupted run.
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as o
from tests import goldens

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "pfcsieve_gb300", "bin", "pfcsieve")
THREADS = str(min(os.cpu_count() or 1, 128))


@pytest.fixture(scope="module", autouse=True)
def built():
    from pfcsieve_gb300 import build
    build.build()


def flags(mode):
    return {1: ["-!"], 2: ["-#"], 4: ["-c"], 5: ["-!", "-c"]}[mode]


def read_factors(path):
    lines = open(path).read().splitlines()
    assert lines, "empty factors.txt"
    checksum = lines[-1]
    body = lines[:-1]
    if body and body[-1] == "no factors":
        body = body[:-1]
    return sorted(body), checksum


def oracle_lines(facs):
    sym = {0: "!", 1: "#", 2: "!/#"}
    out = []
    for f in facs:
        n = abs(int(f["nc"]))
        out.append("%d | %d%s%+d" % (int(f["p"]), n, sym[int(f["type"])], -1 if f["nc"] < 0 else 1))
    return sorted(out)


def test_factors_file_matches_oracle(tmp_path):
    c = goldens.case(3)
    args = flags(c["mode"]) + ["-n", str(c["nmin"]), "-N", str(c["nmax"]), "-p", str(c["pmin"]),
                               "-P", str(c["pmax"]), "-v", THREADS]
    r = subprocess.run([CLI] + args, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    body, checksum = read_factors(tmp_path / "factors.txt")
    assert checksum == c["checksum"]
    _, ofac = o.job(c["mode"], c["nmin"], c["nmax"], c["pmin"], c["pmax"], os.cpu_count() or 1)
    assert body == oracle_lines(ofac)
    assert "factors %d, prime count %d, checksum %s" % (c["factors"], c["primecount"], c["checksum"]) in r.stdout


def test_self_test_passes(tmp_path):
    r = subprocess.run([CLI, "-s", "-v", THREADS], cwd=tmp_path, capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "All test cases completed successfully!" in r.stdout
    assert r.stdout.count("passed.") == 16


def test_resume_after_crash(tmp_path):
    args = ["-!", "-c", "-n", "101", "-N", "2000000", "-p", "1000000000", "-P", "1020000000", "-v", THREADS]
    env = dict(os.environ, PFCSIEVE_CHECKPOINT_SECONDS="0", PFCSIEVE_SEGMENT_SPAN="2000000")
    full = tmp_path / "full"
    part = tmp_path / "part"
    full.mkdir()
    part.mkdir()
    r = subprocess.run([CLI] + args, cwd=full, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    want = read_factors(full / "factors.txt")

    # a host-side crash right after the second checkpoint (no kernel in flight)
    r = subprocess.run([CLI] + args, cwd=part, env=dict(env, PFCSIEVE_EXIT_AFTER_CHECKPOINT="2"),
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 3, r.stdout[-2000:] + r.stderr[-2000:]
    assert r.stdout.count("Checkpoint, current p:") == 2
    assert (part / "stateA.ckp").exists() and (part / "stateB.ckp").exists()

    r = subprocess.run([CLI] + args, cwd=part, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Resuming from checkpoint" in r.stdout
    assert read_factors(part / "factors.txt") == want
