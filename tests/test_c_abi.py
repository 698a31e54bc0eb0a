"""The C ABI from C: tests/c_abi_host.c, a C99 caller of include/pfcsieve.h
compiled with warnings as errors and linked against libpfcsieve.so, runs its
host-only checks (no GPU)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_caller_compiles_links_and_runs(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    from pfcsieve_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "c_abi_host")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c_abi_host.c"),
                        "-L" + libdir, "-lpfcsieve", "-Wl,-rpath," + libdir, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
