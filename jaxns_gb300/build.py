"""In-tree build of libgbns.so with nvcc for sm_103a (no CMake, no torch extension).

Translation units compile in parallel; the link step produces ``jaxns_gb300/_lib/libgbns.so``.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

_HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(_HERE, "csrc")
OUT_DIR = os.path.join(_HERE, "_lib")
OBJ_DIR = os.path.join(os.path.dirname(_HERE), "_build", "obj")
SOURCES = ["gbns_slice.cu", "gbns_slice_warp.cu", "gbns_ns.cu", "gbns_results.cu", "gbns_phiw.cu", "gbns_phiw_tc.cu", "gbns_api.cu",
           "gbns_static.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# Translation units whose fp32 arithmetic is reproduced bit for bit by a CPU model of the
# kernels: no implicit multiply-add contraction, so every fused multiply-add is an explicit
# fmaf in the source and the rounding sequence is the one written there.
EXACT_FP32 = {"gbns_slice.cu", "gbns_slice_warp.cu", "gbns_ns.cu"}


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _deps_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(os.path.dirname(_HERE), "include", "gbns.h"))
    return max(os.path.getmtime(p) for p in paths)


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    lib = os.path.join(OUT_DIR, "libgbns.so")
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _deps_mtime():
        return lib
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        extra = ["-fmad=false"] if src in EXACT_FP32 else []
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + f".tmp{os.getpid()}"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib
