"""The pfcsieve command line: option rules, number suffixes, messages and
checkpoint handling, which all run before the GPU is touched (no GPU needed).

The checkpoint record is the reference's workStatus (cl_sieve.h:14-18) byte
for byte: 8 x u64, 2 x u32, 3 x bool, padded to 80 bytes.
"""
import os
import struct
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "pfcsieve_gb300", "bin", "pfcsieve")


@pytest.fixture(scope="module", autouse=True)
def built():
    from pfcsieve_gb300 import build
    build.build()
    assert os.path.exists(CLI)


def run(args, cwd):
    r = subprocess.run([CLI] + args, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True, timeout=120)
    return r.returncode, r.stdout, r.stderr


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def state(pmin, pmax, p, checksum, primecount, factorcount, nmin, nmax, f, pr, c, last=7, bad=False):
    s = pmin + pmax + p + checksum + primecount + factorcount + last + nmin + nmax
    s = (s + (1 if bad else 0)) % 2**64
    return struct.pack("<8Q2I3?5x", pmin, pmax, p, checksum, primecount, factorcount, last, s,
                       nmin, nmax, f, pr, c)


def test_record_size():
    assert len(state(1, 2, 3, 4, 5, 6, 7, 8, True, False, False)) == 80


@pytest.mark.parametrize("args,msg", [
    (["-n", "101", "-N", "200", "-p", "1e6", "-P", "2e6"], "-! or -# or -c argument is required"),
    (["-#", "-c", "-n", "101", "-N", "200", "-p", "1e6", "-P", "2e6"], "Select only one test type!"),
    (["-!", "-#", "-n", "101", "-N", "200", "-p", "1e6", "-P", "2e6"], "Select only one test type!"),
    (["-!", "-n", "101", "-N", "200"], "-p and -P arguments are required"),
    (["-!", "-p", "1e6", "-P", "2e6"], "-n and -N arguments are required"),
    (["-!", "-n", "300", "-N", "200", "-p", "1e6", "-P", "2e6"], "nmin <= nmax is required"),
    (["-!", "-n", "101", "-N", "200", "-p", "3e6", "-P", "2e6"], "pmin <= pmax is required"),
    (["-!", "-n", "100", "-N", "200", "-p", "1e6", "-P", "2e6"], "out of range argument -n 100"),
    (["-!", "-n", "101", "-N", "2147483648", "-p", "1e6", "-P", "2e6"], "out of range argument -N"),
    (["-!", "-n", "101", "-N", "200", "-p", "2", "-P", "2e6"], "out of range argument -p 2"),
    (["-!", "-n", "101", "-N", "200", "-p", "1x", "-P", "2e6"], "invalid argument -p 1x"),
    (["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "2e6", "-v", "129"], "out of range argument -v"),
    (["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "18447P"], "out of range argument -P 18447P"),
    (["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "1k1"], "invalid argument -P 1k1"),
    (["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "16b60"], "out of range argument -P 16b60"),
    (["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "2e6x"], "invalid argument -P 2e6x"),
    (["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "18446744073709551616"], "out of range argument -P"),
])
def test_rejected(tmp_path, args, msg):
    rc, out, err = run(args, tmp_path)
    assert rc != 0
    assert msg in out + err


@pytest.mark.parametrize("arg,val", [
    ("1K", 1000), ("2M", 2000000), ("3e6", 3000000), ("4k", 4096), ("1m", 1 << 20),
    ("1b20", 1 << 20), ("0x10000", 65536), ("7G", 7 * 10**9), ("2t", 2 << 40), ("1P", 10**15),
    ("5E3", 5000), ("3B4", 48), ("0x10K", 16000), ("9e0", 9), ("16p", 1 << 54), ("010", 8),
    ("18446744073709551615", 2**64 - 1), ("15b60", 15 << 60),
])
def test_number_suffixes(tmp_path, arg, val):
    rc, out, err = run(["-!", "-n", "101", "-N", "200", "-p", "3", "-P", arg], tmp_path)
    assert "Stopping sieve at P: %d N: 200" % val in out


def test_help(tmp_path):
    rc, out, _ = run(["-h"], tmp_path)
    assert rc != 0 and "-!\tUse factorial mode" in out


def test_completed_workunit_resumes_without_gpu(tmp_path):
    (tmp_path / "stateA.ckp").write_bytes(
        state(10**6, 2 * 10**6, 2 * 10**6, 0xABCDEF, 70435, 5, 101, 200, True, False, False))
    rc, out, _ = run(["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "2e6"], tmp_path)
    assert rc == 0
    assert "Resuming from checkpoint in stateA.ckp" in out
    assert "Workunit complete." in out


def test_newer_checkpoint_wins(tmp_path):
    (tmp_path / "stateA.ckp").write_bytes(
        state(10**6, 2 * 10**6, 1500000, 1, 2, 3, 101, 200, True, False, False))
    (tmp_path / "stateB.ckp").write_bytes(
        state(10**6, 2 * 10**6, 2 * 10**6, 1, 2, 3, 101, 200, True, False, False))
    rc, out, _ = run(["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "2e6"], tmp_path)
    assert rc == 0 and "Resuming from checkpoint in stateB.ckp" in out and "Workunit complete." in out


@pytest.mark.parametrize("kind,msg", [
    ("checksum", "Checksum error in stateA.ckp"),
    ("params", "Invalid checkpoint file stateA.ckp"),
    ("short", "Cannot parse stateA.ckp"),
])
def test_bad_checkpoint_is_ignored(tmp_path, kind, msg):
    if have_gpu():
        pytest.skip("would start a real search")
    good = state(10**6, 2 * 10**6, 2 * 10**6, 1, 2, 3, 101, 200, True, False, False)
    data = {
        "checksum": state(10**6, 2 * 10**6, 2 * 10**6, 1, 2, 3, 101, 200, True, False, False, bad=True),
        "params": state(10**6, 3 * 10**6, 2 * 10**6, 1, 2, 3, 101, 200, True, False, False),
        "short": good[:40],
    }[kind]
    (tmp_path / "stateA.ckp").write_bytes(data)
    (tmp_path / "factors.txt").write_text("old\n")
    rc, out, err = run(["-!", "-n", "101", "-N", "200", "-p", "1e6", "-P", "2e6"], tmp_path)
    assert msg in out + err
    # fell back to a fresh start: the results file was truncated, then the GPU was needed
    assert (tmp_path / "factors.txt").read_text() == ""
    assert rc != 0 and "no usable CUDA device" in out + err


@pytest.mark.parametrize("xml,dev", [
    (None, 0),
    ("<app_init_data>\n<gpu_device_num>5</gpu_device_num>\n</app_init_data>\n", 5),
    ("<app_init_data>\n<gpu_type>NVIDIA</gpu_type>\n</app_init_data>\n", 0),
])
def test_init_data_selects_the_device(tmp_path, xml, dev):
    """A BOINC client names the GPU in init_data.xml (<gpu_device_num>,
    main.cpp:252-274); without the file, or without the tag, device 0 is
    used.  The choice is printed before the GPU is touched."""
    if xml is not None:
        (tmp_path / "init_data.xml").write_text(xml)
    rc, out, err = run(["-!", "-n", "101", "-N", "110", "-p", "1000", "-P", "1100"], tmp_path)
    if xml is None:
        assert "init_data.xml not found, using device 0." in out
    else:
        assert "init_data.xml found, using device %d." % dev in out
