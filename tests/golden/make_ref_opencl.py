"""Write tests/golden/ref_opencl_cfg1_factors.txt and ..._cfg2_factors.txt:
the factors.txt files that the reference's own OpenCL program writes for two
of the benchmark searches, run on a GPU.

    python tests/golden/make_ref_opencl.py

Needs oracle/_ref/pfcsieve_ref (oracle/Makefile `stage` then `refcl`) and an
OpenCL-capable GPU (the program checks its OpenCL entry points first with
oracle/_ref/refcl_check).  The files are committed so that the tests compare
against the reference's output on machines without it.
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "pfcsieve_ref")
CHECK = os.path.join(ROOT, "oracle", "_ref", "refcl_check")

SEARCHES = {
    "cfg1": ["-!", "-n", "101", "-N", "20000", "-p", "10000000", "-P", "11000000"],
    "cfg2": ["-!", "-c", "-n", "101", "-N", "200000", "-p", "1000000000", "-P", "1100000000"],
}


def main():
    if not (os.path.exists(EXE) and os.path.exists(CHECK)):
        raise SystemExit("oracle/_ref/pfcsieve_ref not built")
    subprocess.check_call([CHECK])
    threads = str(os.cpu_count() or 2)
    for name, args in SEARCHES.items():
        with tempfile.TemporaryDirectory() as d:
            r = subprocess.run([EXE] + args + ["-v", threads], cwd=d, stdout=subprocess.PIPE, text=True)
            if r.returncode != 0:
                raise SystemExit("%s: reference program failed (%d)" % (name, r.returncode))
            out = os.path.join(HERE, "ref_opencl_%s_factors.txt" % name)
            shutil.copyfile(os.path.join(d, "factors.txt"), out)
            print(name, r.stdout.strip().splitlines()[-1], "->", out)


if __name__ == "__main__":
    sys.exit(main())
