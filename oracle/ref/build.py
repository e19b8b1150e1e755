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

The same kernel translation units are also compiled for the GPU (build_gpu): nvcc, device code only, into one
cubin per translation unit for sm_103a (oracle/_ref/ref_*.cubin), with the reference's own CUDA options
(cmake/Cuda.cmake: C++20, --expt-relaxed-constexpr, --extended-lambda, ptxas -O3; default FMA contraction), and a
probe of the byte layout of the structs its kernels take by value (ref_layout_probe.cpp -> oracle/_ref/
ref_layout.json). oracle/ref_cuda.py loads the cubins through the CUDA driver API and runs the reference's plain
step on the GPU: cubins are device code, so they run on the GPU host although they are built here.

Outputs go to oracle/_ref/ only (git-ignored). Nothing here is built where the reference checkout is absent (the GPU
host): tests that need the library skip there, and what was built here is kept.
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
    return any(os.path.getmtime(f) > t for f in _sources() + OWN_HEADERS + [__file__])


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
    # -Bsymbolic: the library's own CUDA runtime stand-ins (cudaMalloc, cudaMemcpy, ...) must bind inside it even
    # when a process has already loaded the real CUDA runtime globally (torch does), which would otherwise interpose
    r = subprocess.run([os.environ.get("CXX", "g++"), "-shared", "-fopenmp", "-Wl,-Bsymbolic", "-o", tmp, *objs],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    shutil.rmtree(os.path.join(OUT, "obj"), ignore_errors=True)
    return LIB


# ------------------------------------------------------------------ the reference's kernels for the GPU
GPU_SOURCES = {
    "algorithm": "cuda/src/algorithm/Algorithm.cu",
    "boundary": "cuda/src/algorithm/BoundaryAlgorithm.cu",
    "neighbors": "cuda/src/algorithm/neighbors/NeighborKernels.cu",
}
GPU_ARCH = "-gencode=arch=compute_103a,code=sm_103a"
LAYOUT = os.path.join(OUT, "ref_layout.json")
PROBE = os.path.join(HERE, "ref_layout_probe.cpp")


def cubin_path(name: str) -> str:
    return os.path.join(OUT, f"ref_{name}.cubin")


def gpu_outputs():
    return [cubin_path(k) for k in GPU_SOURCES] + [LAYOUT]


def _nvcc() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return os.path.join(cand, "bin", "nvcc")
    return "nvcc"


def _cubin(item):
    name, rel = item
    root = reference_root()
    out = cubin_path(name)
    cmd = [_nvcc(), "-cubin", GPU_ARCH, "-std=c++20", "--expt-relaxed-constexpr", "--extended-lambda",
           "-diag-suppress", "20012", "-O3", "--ptxas-options=-O3", "-DGLM_ENABLE_EXPERIMENTAL", "-w",
           "-I", os.path.join(HERE, "glm_api"), "-I", os.path.join(root, "cuda", "src"),
           "-I", os.path.join(root, "cuda", "include"), os.path.join(root, rel), "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {rel}:\n{r.stdout}\n{r.stderr[-4000:]}")
    os.replace(out + ".tmp", out)
    return out


def _layout():
    exe = os.path.join(OUT, "ref_layout_probe")
    flags = [f for f in _flags() if f != "-fopenmp"]
    cmd = [os.environ.get("CXX", "g++"), *flags, "-include", "algorithm/WendlandKernel.cuh", "-x", "c++", PROBE,
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"layout probe build failed:\n{r.stderr[-4000:]}")
    r = subprocess.run([exe], capture_output=True, text=True, check=True)
    with open(LAYOUT + ".tmp", "w") as f:
        f.write(r.stdout)
    os.replace(LAYOUT + ".tmp", LAYOUT)
    os.remove(exe)
    return LAYOUT


def gpu_needs_build() -> bool:
    outs = gpu_outputs()
    if not all(os.path.exists(o) for o in outs):
        return True
    t = min(os.path.getmtime(o) for o in outs)
    srcs = [os.path.join(reference_root(), s) for s in GPU_SOURCES.values()] + OWN_HEADERS + [PROBE, __file__]
    return any(os.path.getmtime(f) > t for f in srcs)


def build_gpu(force: bool = False):
    """Builds the reference's kernels for the GPU (cubins) and their argument layout, where the reference checkout
    is present; returns the output paths that exist (those built earlier are kept where the checkout is absent)."""
    if available() and (force or gpu_needs_build()):
        os.makedirs(OUT, exist_ok=True)
        with cf.ThreadPoolExecutor(max_workers=len(GPU_SOURCES) + 1) as ex:
            futs = [ex.submit(_cubin, it) for it in GPU_SOURCES.items()] + [ex.submit(_layout)]
            for f in futs:
                f.result()
    return [o for o in gpu_outputs() if os.path.exists(o)]


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_gpu(force="--force" in sys.argv))
