"""Builds libosgpu.so (the C ABI of include/osgpu.h) for sm_103a, in tree.

Each translation unit is compiled by nvcc in parallel, then linked with the
static CUDA runtime.  Host code is compiled with -ffp-contract=off so the
sampling analysis rounds exactly like the reference (no fused multiply-add).
"""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
# OSGPU_LIB_DIR / OSGPU_NVCC_FLAGS build side-by-side variants (tuning runs).
OUT_DIR = os.environ.get("OSGPU_LIB_DIR") or os.path.join(HERE, "lib")
LIB = os.path.join(OUT_DIR, "libosgpu.so")
SOURCES = ["prop_kernels.cu", "prop_fast.cu", "api.cu", "host_analysis.cpp", "noalloc.cu",
           "inverse_kernels.cu", "gs_fast.cu"]
HEADERS = ["fft_smem.cuh", "fft_reg.cuh", "elements.cuh", "prop_kernels.cuh", "osgpu_types.h",
           "host_analysis.h", "inverse_kernels.cuh",
           "gs_fast.cuh", "tma.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                "-I" + os.path.join(ROOT, "include")] + os.environ.get("OSGPU_NVCC_FLAGS", "").split()


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(ROOT, "include", "osgpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile every CUDA/C++ source of the library; returns the .so path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src + ".o")
        cmd = [nvcc] + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
