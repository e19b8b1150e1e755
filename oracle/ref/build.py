"""Build recipe of the reference checker (TEST INFRASTRUCTURE ONLY): AdaptiveSph's own kernels compiled as host C++
into oracle/_ref/libasph_ref_host.so.

The reference's translation units are compiled unchanged from where they lie (the reference checkout, by default
/root/reference, or $ASPH_REFERENCE_ROOT) with g++ and OpenMP: the kernels (cuda/src/algorithm/Algorithm.cu,
BoundaryAlgorithm.cu, AdaptiveAlgorithm.cu, algorithm/neighbors/NeighborKernels.cu) and the boundary generator
(cuda/src/simulation/physics/StaticBoundaryDomain.cu), together with ref_host_run.cpp (the launcher and the host
orchestration restated from the reference's class files). The two third-party libraries the reference fetches with
CMake and that are absent here are replaced by restatements of the parts of their APIs it uses: glm 1.0.1
(glm_api/) and nanoflann 1.8.0 (nanoflann_api/). CUDA's own headers supply the vector types; host_cuda/ supplies the
thread coordinates and atomics that nvcc would. Thrust runs on its CPP (host) system. No CMake, no generated code.

Outputs go to oracle/_ref/ only (git-ignored). Nothing here is built where the reference checkout is absent (the GPU
box): tests that need the library skip there.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libasph_ref_host.so")
REF_SOURCES = [
    "cuda/src/algorithm/Algorithm.cu",
    "cuda/src/algorithm/BoundaryAlgorithm.cu",
    "cuda/src/algorithm/AdaptiveAlgorithm.cu",
    "cuda/src/algorithm/neighbors/NeighborKernels.cu",
    "cuda/src/simulation/physics/StaticBoundaryDomain.cu",
]
OWN_SOURCES = [os.path.join(HERE, "ref_host_run.cpp")]
OWN_HEADERS = [os.path.join(HERE, d, f) for d in ("glm_api/glm", "glm_api/glm/ext", "glm_api/glm/gtx", "nanoflann_api",
                                                   "host_cuda")
               for f in (os.listdir(os.path.join(HERE, d)) if os.path.isdir(os.path.join(HERE, d)) else [])
               if f.endswith((".h", ".hpp"))]


def reference_root() -> str:
    return os.environ.get("ASPH_REFERENCE_ROOT", "/root/reference")


def available() -> bool:
    root = reference_root()
    return all(os.path.exists(os.path.join(root, s)) for s in REF_SOURCES)


def _cuda_include() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "vector_types.h")):
            return os.path.join(cand, "include")
    raise RuntimeError("CUDA headers not found")


def _flags():
    root = reference_root()
    inc = _cuda_include()
    return ["-std=c++20", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-w",
            "-include", os.path.join(HERE, "host_cuda", "asph_ref_host_prelude.h"),
            "-I", os.path.join(HERE, "host_cuda"), "-I", os.path.join(HERE, "glm_api"),
            "-I", os.path.join(HERE, "nanoflann_api"), "-I", ORACLE,
            "-I", os.path.join(root, "cuda", "src"), "-I", os.path.join(root, "cuda", "include"),
            "-I", inc, "-I", os.path.join(inc, "cccl"),
            "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP"]


def _sources():
    root = reference_root()
    return [os.path.join(root, s) for s in REF_SOURCES] + OWN_SOURCES


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _sources() + OWN_HEADERS)


def _compile(src: str) -> str:
    obj = os.path.join(OUT, "obj", os.path.basename(src).replace(".", "_") + ".o")
    cmd = [os.environ.get("CXX", "g++"), *_flags(), "-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for {src}:\n{r.stdout}\n{r.stderr[-4000:]}")
    return obj


def build(force: bool = False):
    """Builds the library if the reference checkout is present; returns its path, or None without the checkout."""
    if not available():
        return LIB if os.path.exists(LIB) else None
    if not force and not needs_build():
        return LIB
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(_sources())) as ex:
        objs = list(ex.map(_compile, _sources()))
    tmp = LIB + ".tmp"
    r = subprocess.run([os.environ.get("CXX", "g++"), "-shared", "-fopenmp", "-o", tmp, *objs],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    shutil.rmtree(os.path.join(OUT, "obj"), ignore_errors=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
