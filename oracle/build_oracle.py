"""Build the CPU oracle ``oracle/_build/libptoracle.so`` (test infrastructure).

The oracle is plain C.  It is compiled with -ffp-contract=off and without fast-math
so its single-precision lookups round like the reference's.  OpenMP parallelises only
the per-person schedule generation; every result is independent of the thread count.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libptoracle.so")
    src = os.path.join(HERE, "pt_oracle.c")
    hdr = os.path.join(HERE, "pt_oracle.h")
    if os.path.exists(so) and os.path.getmtime(so) >= max(os.path.getmtime(src), os.path.getmtime(hdr)):
        return so
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", "-Wall", "-o", so, src, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return so


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
