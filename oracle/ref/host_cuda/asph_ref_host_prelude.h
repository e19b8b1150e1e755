// asph_ref_host_prelude.h — force-included when the reference's CUDA translation units are compiled as host C++ for
// the CPU checker (TEST INFRASTRUCTURE ONLY: it builds oracle/_ref). It supplies what nvcc would: the thread
// coordinates of the kernel being emulated (set per emulated thread by the launcher in ref_host_run.cpp) and the
// atomic operations (device_atomic_functions.h in this directory).
#pragma once

#include <cuda_runtime.h>

namespace asph_ref_host {
struct Coord {
    unsigned int x, y, z;
};
}  // namespace asph_ref_host

extern thread_local asph_ref_host::Coord threadIdx;
extern thread_local asph_ref_host::Coord blockIdx;
extern thread_local asph_ref_host::Coord blockDim;
extern thread_local asph_ref_host::Coord gridDim;

#include "device_atomic_functions.h"
