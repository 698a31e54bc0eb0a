"""Build the CUDA library (libpfcsieve.so) and the pfcsieve CLI in-tree.

Kernels are compiled for sm_103a only (GB300).  Outputs:
    pfcsieve_gb300/lib/libpfcsieve.so
    pfcsieve_gb300/bin/pfcsieve
Object files go to pfcsieve_gb300/_build/.  Steps run in parallel and are
skipped when their outputs are newer than every source and header.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libpfcsieve.so")
CLI = os.path.join(BINDIR, "pfcsieve")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp", "-I" + INC, "-I" + CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-I" + INC, "-I" + CSRC]

CU_SOURCES = ["gen.cu", "sieve.cu", "setup_tc.cu", "api.cu", "batch.cu", "verify.cu", "peak.cu", "noalloc.cu"]
CXX_SOURCES = ["host.cpp"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pfcsieve_gb300")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        glob.glob(os.path.join(INC, "*.h"))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(force=False, verbose=False, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            extra = ["-Xptxas", "-v"] if ptxas_verbose else []
            jobs.append([nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    for s in CXX_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    outs = []
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for o in ex.map(lambda c: _run(c, verbose), jobs):
            outs.append(o)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs +
             ["-Xcompiler", "-fopenmp", "-lgomp"], verbose)
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB] + hdrs)):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + INC, cli_src, "-o", CLI,
              "-L" + LIBDIR, "-lpfcsieve", "-Wl,-rpath,$ORIGIN/../lib", "-fopenmp"], verbose)
    if ptxas_verbose:
        return "".join(outs)
    return LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    out = build(force=force, verbose=True, ptxas_verbose="--ptxas" in sys.argv)
    print(out)
