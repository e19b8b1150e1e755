// boundary_internal.h — wall generation on the device (boundary_kernels.cu) shared with the simulation runtime
// (simulation.cu); not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/asph.h"

namespace asph {

// Wall particles generated on the device: positions (w = 0) and psi, in the reference's order.
struct DeviceWalls {
    float4* pos = nullptr;
    float* psi = nullptr;
    float* seq = nullptr;  // the lattice's coordinate sequences
    uint32_t n = 0;
    uint32_t launches = 0;
};

// StaticBoundaryDomain::generate (StaticBoundaryDomain.cu:76-174) on `stream`; returns after the walls are ready.
asph_status generate_walls_device(const asph_domain& d, float spacing, float rho0, float h, cudaStream_t stream,
                                  DeviceWalls& out);
void free_walls(DeviceWalls& w);

// the library's error reporting (simulation.cu): records the message returned by asph_last_error()
asph_status report_error(asph_status s, const std::string& msg);
asph_status report_cuda_error(cudaError_t e, const char* what);

}  // namespace asph
