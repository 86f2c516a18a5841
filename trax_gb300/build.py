"""Builds libtrax_gb300.so (sm_103a) in-tree with nvcc.

FP32 contract shared with the CPU oracle (trax_math.h): device code without
FMA contraction, IEEE division and square root, no flush-to-zero; host code
with -ffp-contract=off.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libtrax_gb300.so")
SOURCES = [os.path.join(CSRC, f) for f in ("trax_capi.cu", "trax_serve.cpp", "trax_pb.cpp",
                                           "trax_physics.cpp")]
DEPS = SOURCES + [os.path.join(CSRC, f) for f in ("trax_kernels.cuh", "trax_ingest.cuh",
                                                   "trax_physics.cuh", "trax_math.h")] + [
    os.path.join(HERE, "..", "include", "trax.h")]

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [
    ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
    "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-shared", "-cudart=static",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in DEPS if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    if not force and up_to_date():
        return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *NVCC_FLAGS, "-Xcompiler", "-pthread", *extra, "-o", tmp, *SOURCES]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd, cwd=HERE)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    extra = [a for a in sys.argv[1:] if a.startswith("-")]
    print(build(force=True, verbose=True, extra=extra))
