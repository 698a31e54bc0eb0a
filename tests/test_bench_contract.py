"""bench.py's reference arm on the host cores, no GPU: the JSON line's
contract (keys, units, the cpu_baseline and e2e objects of a CPU arm), and
under torchrun with two ranks one line from rank 0 while the other rank exits
without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _lines(out):
    return [json.loads(x) for x in out.splitlines() if x.startswith("{")]


def _run(cmd, timeout=600):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def test_reference_arm_line():
    r = _run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "0",
              "--cpu-sample", "2000"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    if "unavailable" in d:
        pytest.skip(d["unavailable"])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "(p,n) pairs tested/s" and d["unit"] == "pairs/s"
    assert d["steps"] == 2 and d["warmup"] == 0 and d["n_gpus"] == 1 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "-! -c n=[101,200000) p=[1e9,1.1e9)"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["unit"] == "pairs/s" and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    r = _run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
              "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
              "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-sample", "1000"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference"
