"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/nsmp_oracle.cpp into oracle/_build/libnsmp_oracle.so with
g++ and OpenMP.  FMA contraction is disabled so each floating-point
operation rounds exactly as the Fortran reference's unfused arithmetic.
The reference itself (Fortran 90 + MPI) cannot be built here: no Fortran
compiler exists in this image or on the GPU machine, so oracle/_ref stays empty.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nsmp_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnsmp_oracle.so")


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "nsmp_oracle.h")]
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-o", LIB + ".tmp", SRC]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
