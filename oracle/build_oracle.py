"""Builds the CPU oracle (test infrastructure) into oracle/_build/.

g++ with OpenMP and -ffp-contract=off (no fused multiply-add, so the FP64
oracle rounds every operation exactly as written).  The reference itself is
Fortran 90 + MPI and no Fortran compiler is available, so there is no
oracle/_ref build of the reference.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmc_oracle.so")


SOURCES = ("mc_oracle.cpp", "update_oracle.cpp")


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    hdr = os.path.join(os.path.dirname(HERE), "include", "mocassin_gpu.h")
    newest = max([os.path.getmtime(s) for s in srcs] + [os.path.getmtime(hdr)])
    if force or not os.path.exists(LIB) or newest > os.path.getmtime(LIB):
        cmd = ["g++", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c++17", "-o", LIB] + srcs
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + p.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
