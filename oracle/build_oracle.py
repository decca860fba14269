"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/fk_oracle.cpp into oracle/_build/liboracle.so with the host
g++ (plain -O3, no -march flags, so the same recipe works on x86_64 and
aarch64). The reference itself cannot be compiled here: it needs Eigen3,
Boost.MPI, ALPSCore, ARPACK, FFTW, gftools and HDF5, none of which is
installed, so there is no oracle/_ref build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fk_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-pthread", "-o", LIB + ".tmp", SRC]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
