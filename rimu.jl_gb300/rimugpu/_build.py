"""Build of librimu_gpu.so: nvcc for sm_103a only, one object per translation unit in
parallel, then a shared-library link.  Output stays in-tree under ``rimu.jl_gb300/_build``."""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # rimu.jl_gb300/
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "librimu_gpu.so")
SOURCES = ["fciqmc.cu", "hv.cu", "capi.cu", "batch.cu", "vecops.cu"]
HEADERS = ["rimu_device.cuh", "rimu_internal.h"]
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no implicit multiply-add contraction, so every float expression rounds as
# written (the kernels request fused multiply-adds explicitly where they want them).
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC"]


def _newest_input() -> float:
    paths = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    paths.append(os.path.join(os.path.dirname(PKG), "include", "rimu_gpu.h"))
    return max(os.path.getmtime(p) for p in paths)


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [NVCC, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB
