"""Build recipe for the C++ oracle: oracle/_build/libtbl_oracle.so.

g++ only, no build system.  -ffp-contract=off keeps the Fortran expression
order without fused multiply-adds; -fopenmp parallelises the per-slab loops
without changing results (reductions are combined in rank order).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtbl_oracle.so")
SRC = os.path.join(HERE, "tbl_oracle.cpp")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
