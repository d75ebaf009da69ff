"""Build recipe of libamr_gb300.so (sm_103a).

Compiles every translation unit under csrc/ in parallel (nvcc for .cu, g++ for .cpp) into
csrc/_build/ and links adaptivemesh_gb300/libamr_gb300.so against the shared CUDA runtime.
Incremental: a unit is rebuilt when it or any header under csrc/ or include/ is newer than
its object.

Device code is compiled with -fmad=false (the kernels spell out every fused multiply-add) and
-ftz=true (subnormals flush to zero, as in the reference's fast-math build), except the units listed
in CONTRACTED; host code with -ffp-contract=off, so host float arithmetic rounds the same on x86-64
and aarch64.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(CSRC, "_build")
LIB = os.path.join(PKG, "libamr_gb300.so")
INCLUDE = os.path.join(ROOT, "include")


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-fmad=false", "-ftz=true", "-prec-div=true",
              "-prec-sqrt=true", "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
              "-I", INCLUDE, "-I", CSRC]
# Units without a reference build to reproduce bit for bit (the evolutions, held to an FP64 oracle
# within stated tolerances) let the compiler contract products and sums into fused multiply-adds.
CONTRACTED = {"kernels_evolve.cu", "estimator.cu"}
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _compile(src: str, newest_header: float) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), newest_header):
        return obj
    if src.endswith(".cu"):
        flags = NVCC_FLAGS
        if os.path.basename(src) in CONTRACTED:
            flags = [("-fmad=true" if f == "-fmad=false" else f) for f in NVCC_FLAGS]
        cmd = [_nvcc(), *flags, "-c", src, "-o", obj + ".tmp"]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-I", os.path.join(os.path.dirname(_nvcc()), "..", "include"),
               "-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    """Compile and link libamr_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    newest = max(os.path.getmtime(h) for h in _headers())
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, newest), sources))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", LIB + ".tmp", *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
