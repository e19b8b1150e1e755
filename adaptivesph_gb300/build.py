"""Builds libasph_gb300.so in-tree: hand-written CUDA for sm_103a plus the host runtime, behind the C ABI of
include/asph.h.

nvcc compiles each .cu for ``-gencode arch=compute_103a,code=sm_103a`` with ``-fmad=false`` (the kernels spell out
every fused multiply-add they want) and g++ compiles the host-only .cpp; translation units build in parallel.
The CUDA runtime is linked statically, so the library needs only the driver at run time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libasph_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CU_SOURCES = ["step_kernels.cu", "neighbor_kernels.cu", "refine_kernels.cu", "radix_sort.cu", "boundary_kernels.cu",
              "simulation.cu"]
CPP_SOURCES = ["boundary_domain.cpp", "server.cpp"]
HEADERS = ["asph_device.cuh", "asph_kernels.cuh", "asph_refine.cuh", "batch_internal.h", "boundary_internal.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES + HEADERS]
    files.append(os.path.join(INCLUDE, "asph.h"))
    return files


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def _compile_cu(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [_nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", CSRC, "-I", INCLUDE, "-rdc=false", "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def _compile_cpp(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-I", INCLUDE,
           "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compiles the library if any source is newer than it; returns its path."""
    if not force and not verbose_ptxas and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(CU_SOURCES) + len(CPP_SOURCES)) as ex:
        futs = [ex.submit(_compile_cu, s, verbose_ptxas) for s in CU_SOURCES]
        futs += [ex.submit(_compile_cpp, s) for s in CPP_SOURCES]
        objs = [f.result() for f in futs]
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
