// ref_layout_probe.cpp — prints, as JSON, the byte layout of the structs that AdaptiveSph's kernels take by value
// (TEST INFRASTRUCTURE ONLY: built and run by oracle/ref/build.py where the reference checkout exists; its output,
// oracle/_ref/ref_layout.json, lets oracle/ref_cuda.py pack kernel arguments for the reference's kernels compiled
// for the GPU without the reference's headers, which the GPU host does not have).
//
// Structs (reference file:line): FluidParticlesData and BoundaryParticlesData (cuda/include/cuda/simulation/
// Simulation.cuh:22-44), Simulation::Parameters and its Domain (Simulation.cuh:64-109), NeighborGrid::Grid,
// GridData and Device (cuda/src/simulation/neighbors/NeighborGrid.cuh:12-46). std::span<int32_t> is a pointer and
// a size_t in the standard library both host compilers use (libstdc++); the probe records where each lies by
// writing a known span and finding its bytes, so nothing about its layout is assumed. The host (x86-64 here,
// aarch64 on the GPU host) and the device share these layouts: LP64, natural alignment, no packing pragmas.
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "algorithm/neighbors/NeighborKernels.cuh"

thread_local asph_ref_host::Coord threadIdx{0, 0, 0};
thread_local asph_ref_host::Coord blockIdx{0, 0, 0};
thread_local asph_ref_host::Coord blockDim{1, 1, 1};
thread_local asph_ref_host::Coord gridDim{1, 1, 1};

using namespace sph::cuda;

namespace {

// Offset of a span's data pointer and size inside an object of type T, found by writing a distinctive span into
// a zeroed object and searching its bytes.
template <class T, class Set>
void span_offsets(Set set, size_t& ptr_off, size_t& size_off) {
    alignas(T) unsigned char buf[sizeof(T)];
    std::memset(buf, 0, sizeof(T));
    T* obj = reinterpret_cast<T*>(buf);
    int32_t* marker = reinterpret_cast<int32_t*>(uintptr_t(0x1122334455667700ull));
    const size_t count = 0x0a0b0c0d0e0full;
    set(*obj, std::span<int32_t>(marker, count));
    ptr_off = size_off = SIZE_MAX;
    for (size_t o = 0; o + 8 <= sizeof(T); o += 8) {
        uint64_t v;
        std::memcpy(&v, buf + o, 8);
        if (v == uint64_t(uintptr_t(marker))) ptr_off = o;
        if (v == count) size_off = o;
    }
}

void field(const char* name, size_t off, bool last = false) { std::printf("    \"%s\": %zu%s\n", name, off, last ? "" : ","); }

}  // namespace

int main() {
    std::printf("{\n");
    std::printf("  \"FluidParticlesData\": {\n    \"size\": %zu,\n", sizeof(FluidParticlesData));
    field("positions", offsetof(FluidParticlesData, positions));
    field("velocities", offsetof(FluidParticlesData, velocities));
    field("accelerations", offsetof(FluidParticlesData, accelerations));
    field("densities", offsetof(FluidParticlesData, densities));
    field("radii", offsetof(FluidParticlesData, radii));
    field("smoothingRadii", offsetof(FluidParticlesData, smoothingRadii));
    field("masses", offsetof(FluidParticlesData, masses));
    field("particleCount", offsetof(FluidParticlesData, particleCount), true);
    std::printf("  },\n");

    std::printf("  \"BoundaryParticlesData\": {\n    \"size\": %zu,\n", sizeof(BoundaryParticlesData));
    field("positions", offsetof(BoundaryParticlesData, positions));
    field("colors", offsetof(BoundaryParticlesData, colors));
    field("psiValues", offsetof(BoundaryParticlesData, psiValues));
    field("viscosityCoefficients", offsetof(BoundaryParticlesData, viscosityCoefficients));
    field("radii", offsetof(BoundaryParticlesData, radii));
    field("particleCount", offsetof(BoundaryParticlesData, particleCount), true);
    std::printf("  },\n");

    using P = Simulation::Parameters;
    using D = P::Domain;
    std::printf("  \"Domain\": {\n    \"size\": %zu,\n", sizeof(D));
    field("min", offsetof(D, min));
    field("max", offsetof(D, max));
    field("friction", offsetof(D, friction), true);
    std::printf("  },\n");
    std::printf("  \"Parameters\": {\n    \"size\": %zu,\n", sizeof(P));
    field("domain", offsetof(P, domain));
    field("gravity", offsetof(P, gravity));
    field("speedOfSound", offsetof(P, speedOfSound));
    field("restDensity", offsetof(P, restDensity));
    field("restitution", offsetof(P, restitution));
    field("viscosityConstant", offsetof(P, viscosityConstant));
    field("surfaceTensionConstant", offsetof(P, surfaceTensionConstant));
    field("maxVelocity", offsetof(P, maxVelocity));
    field("baseSmoothingRadius", offsetof(P, baseSmoothingRadius));
    field("baseParticleRadius", offsetof(P, baseParticleRadius));
    field("baseParticleMass", offsetof(P, baseParticleMass));
    field("threadsPerBlock", offsetof(P, threadsPerBlock), true);
    std::printf("  },\n");

    using G = NeighborGrid::Grid;
    std::printf("  \"Grid\": {\n    \"size\": %zu,\n", sizeof(G));
    field("gridSize", offsetof(G, gridSize));
    field("cellSize", offsetof(G, cellSize), true);
    std::printf("  },\n");

    using GD = NeighborGrid::GridData;
    size_t p[4][2];
    span_offsets<GD>([](GD& g, std::span<int32_t> s) { g.cellStartIndices = s; }, p[0][0], p[0][1]);
    span_offsets<GD>([](GD& g, std::span<int32_t> s) { g.cellEndIndices = s; }, p[1][0], p[1][1]);
    span_offsets<GD>([](GD& g, std::span<int32_t> s) { g.particleGridIndices = s; }, p[2][0], p[2][1]);
    span_offsets<GD>([](GD& g, std::span<int32_t> s) { g.particleArrayIndices = s; }, p[3][0], p[3][1]);
    std::printf("  \"GridData\": {\n    \"size\": %zu,\n", sizeof(GD));
    field("cellStartIndices.data", p[0][0]);
    field("cellStartIndices.size", p[0][1]);
    field("cellEndIndices.data", p[1][0]);
    field("cellEndIndices.size", p[1][1]);
    field("particleGridIndices.data", p[2][0]);
    field("particleGridIndices.size", p[2][1]);
    field("particleArrayIndices.data", p[3][0]);
    field("particleArrayIndices.size", p[3][1]);
    field("particleCount", offsetof(GD, particleCount), true);
    std::printf("  },\n");

    using DV = NeighborGrid::Device;
    std::printf("  \"Device\": {\n    \"size\": %zu,\n", sizeof(DV));
    field("domain", offsetof(DV, domain));
    field("grid", offsetof(DV, grid));
    field("fluid", offsetof(DV, fluid));
    field("boundary", offsetof(DV, boundary), true);
    std::printf("  },\n");
    std::printf("  \"wendlandRangeRatio\": %.9g\n", (double)device::constant::wendlandRangeRatio);
    std::printf("}\n");
    return 0;
}
