"""Build libspecter_gpu.so in-tree for sm_103a (GB300) with nvcc, and the CPU oracle library.

    python -m specter_gb300.build          # or: import specter_gb300.build as b; b.build()

Translation units compile in parallel, then link into specter_gb300/libspecter_gpu.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "libspecter_gpu.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["plan.cu", "ops_f64.cu", "ops_f32.cu", "fast_f32.cu", "fast_x_f32.cu", "fast_y_f32.cu", "fused.cu", "fused_ffb.cu", "fused_ffb_pair.cu", "fused_ff_generic.cu", "fused_fast_f32.cu", "fused_small_f32.cu", "noalloc.cu", "capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xcompiler", "-Wno-deprecated-declarations"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _deps_mtime() -> float:
    m = 0.0
    for root in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(root):
            m = max(m, os.path.getmtime(os.path.join(root, f)))
    return m


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link the shared library."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def build_oracle() -> str:
    """Compile the CPU oracle (test infrastructure) with its committed Makefile."""
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    return O.build(force=True)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
