"""Build libgpugo.so (CUDA, sm_103a) in-tree with nvcc.

``--fmad=false`` and ``-ffp-contract=off`` keep every round-to-nearest operation
a separate rounding; the interval bounds depend on it bit for bit.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgpugo.so")
SOURCES = ["engine.cu"]
HEADERS = ["ia.cuh", "families.cuh", "codelist.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "gpugo.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    # ptxas compiles the module's functions on all cores (the same code per
    # function: only the optimisation passes run in parallel)
    cmd = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-shared",
           "-Xptxas", "--split-compile=0",
           "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
           "-o", tmp] + [os.path.join(CSRC, f) for f in SOURCES]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def build_host_asan() -> str:
    """The same library with its host code under AddressSanitizer, for the tests
    of the host-side checks (code lists, checkpoints, arguments) that run without
    a GPU.  The device code is left as PTX (no ptxas pass), which keeps the build
    short; load it with GPUGO_LIB=<path> and LD_PRELOAD=<gcc's libasan.so>."""
    out = os.path.join(OUT_DIR, "asan", "libgpugo.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = [nvcc(), "-gencode=arch=compute_103a,code=compute_103a", "-O1", "-g", "-std=c++17", "--fmad=false",
           "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math,-fsanitize=address,-fno-omit-frame-pointer",
           "-o", out] + [os.path.join(CSRC, f) for f in SOURCES]
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    if "--host-asan" in sys.argv:
        print(build_host_asan())
    else:
        print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
