"""In-tree build of libmcgpu.so (sm_103a) with nvcc, one process per unit.

The FP64 transport unit is compiled with -fmad=false so its arithmetic
matches the FP64 oracle operation for operation; every other unit keeps
contraction on.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(ROOT, "csrc")
LIBDIR = os.path.join(ROOT, "lib")
LIB = os.path.join(LIBDIR, "libmcgpu.so")
OBJDIR = os.path.join(ROOT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]

# (source, extra flags)
UNITS = [
    ("mcgpu_api.cu", []),
    ("transport_fp32.cu", []),
    ("transport_fp64.cu", ["-fmad=false"]),
    ("transport_noalloc.cu", ["-fmad=false"]),
    ("opacity.cu", []),
    ("jmoments.cu", []),
    ("cellupdate.cu", ["-fmad=false", "-Xcompiler=-ffp-contract=off"]),
    ("cellupdate_fp32.cu", []),
    ("mlp.cu", []),
    ("emission.cu", []),
]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stdout + p.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".inc"))]
    headers.append(os.path.join(os.path.dirname(ROOT), "include", "mocassin_gpu.h"))
    jobs, objs = [], []
    for src, extra in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers + [__file__]):
            jobs.append([nvcc()] + ARCH + COMMON + extra + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
