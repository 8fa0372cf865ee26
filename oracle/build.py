"""Build recipe of the CPU oracle (test infrastructure, never the product).

Compiles oracle/mge_oracle.cpp into oracle/_build/libmge_oracle.so with
-O2 -ffp-contract=off so every Fortran expression of the reference rounds as
gfortran -O2 evaluates it without FMA contraction.  OpenMP parallelises only
loops whose iterations are independent, so results do not depend on the
thread count.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libmge_oracle.so")
SRC = os.path.join(HERE, "mge_oracle.cpp")


def build(force=False, verbose=False):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    deps = [SRC, os.path.join(HERE, "mge_oracle.h"), os.path.join(HERE, "..", "include", "mge_gpu.h")]
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(d) for d in deps):
        return OUT
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-Wall", "-Wno-unused-variable", "-Wno-unused-but-set-variable", "-o", OUT + ".tmp", SRC]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
