// asph.hpp — C++ interface over the C ABI of asph.h, shaped like the reference's simulation interface
// (cuda/include/cuda/simulation/Simulation.cuh:61-145, physics/StaticBoundaryDomain.cuh:14-41,
// memory/ImportedMemory.cuh:10-26): the same class and function names, argument order and meaning, with plain
// float[4] positions instead of glm::vec4 and exceptions instead of unchecked CUDA calls. Header only; link
// against libasph_gb300.so.
#ifndef ASPH_HPP
#define ASPH_HPP

#include <array>
#include <cstdint>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

#include "asph.h"

namespace asph {

class Error : public std::runtime_error {
public:
    Error(asph_status status, const std::string& where)
        : std::runtime_error(where + ": " + asph_status_string(status) + " (" + asph_last_error() + ")"),
          status_(status) {}
    asph_status status() const noexcept { return status_; }

private:
    asph_status status_;
};

inline void check(asph_status s, const char* where) {
    if (s != ASPH_OK) throw Error(s, where);
}

using vec4 = std::array<float, 4>;

// ImportedMemory (ImportedMemory.cuh:10-20): a device buffer the simulation writes its particles into.
class ImportedMemory {
public:
    explicit ImportedMemory(asph_memory* m) : m_(m) {}
    ~ImportedMemory() { asph_memory_release(m_); }
    ImportedMemory(const ImportedMemory&) = delete;
    ImportedMemory& operator=(const ImportedMemory&) = delete;
    const asph_memory* handle() const noexcept { return m_; }
    void* data() const {
        void* p = nullptr;
        check(asph_memory_device_pointer(m_, &p), "asph_memory_device_pointer");
        return p;
    }
    size_t size() const {
        size_t n = 0;
        check(asph_memory_size(m_, &n), "asph_memory_size");
        return n;
    }

private:
    asph_memory* m_;
};

// importBuffer(int handle, size_t size) (ImportedMemory.cuh:25)
inline std::unique_ptr<ImportedMemory> importBuffer(int handle, size_t size) {
    asph_memory* m = nullptr;
    check(asph_import_buffer_fd(handle, size, &m), "asph_import_buffer_fd");
    return std::make_unique<ImportedMemory>(m);
}

// Headless stand-in for a buffer exported by the renderer.
inline std::unique_ptr<ImportedMemory> allocateBuffer(size_t size) {
    asph_memory* m = nullptr;
    check(asph_memory_allocate(size, &m), "asph_memory_allocate");
    return std::make_unique<ImportedMemory>(m);
}

// FluidParticlesDataImportedBuffer / BoundaryParticlesDataImportedBuffer (Simulation.cuh:46-59)
struct FluidParticlesDataImportedBuffer {
    const ImportedMemory* positions = nullptr;
    const ImportedMemory* velocities = nullptr;
    const ImportedMemory* densities = nullptr;
    const ImportedMemory* radii = nullptr;
};

struct BoundaryParticlesDataImportedBuffer {
    const ImportedMemory* positions = nullptr;
    const ImportedMemory* radii = nullptr;
    const ImportedMemory* colors = nullptr;
};

// physics::StaticBoundaryDomain (StaticBoundaryDomain.cuh:14-41)
class StaticBoundaryDomain {
public:
    using Particle = asph_boundary_particle;

    static StaticBoundaryDomain generate(const asph_domain& bounds, float particleSpacing, float fluidRestDensity,
                                         float fluidSmoothingRadius) {
        uint32_t n = 0;
        check(asph_boundary_generate(&bounds, particleSpacing, fluidRestDensity, fluidSmoothingRadius, nullptr, 0, &n),
              "asph_boundary_generate");
        std::vector<Particle> particles(n);
        check(asph_boundary_generate(&bounds, particleSpacing, fluidRestDensity, fluidSmoothingRadius,
                                     particles.data(), n, &n),
              "asph_boundary_generate");
        return StaticBoundaryDomain(bounds, std::move(particles));
    }
    const std::vector<Particle>& getParticles() const noexcept { return particles_; }
    uint32_t getParticleCount() const noexcept { return static_cast<uint32_t>(particles_.size()); }
    const asph_domain& bounds() const noexcept { return bounds_; }

private:
    StaticBoundaryDomain(const asph_domain& b, std::vector<Particle> p) : bounds_(b), particles_(std::move(p)) {}
    asph_domain bounds_;
    std::vector<Particle> particles_;
};

// Simulation (Simulation.cuh:61-136). update() also writes the imported buffers, as the reference's update does.
class Simulation {
public:
    using Parameters = asph_parameters;
    using DensityInfo = asph_density_info;

    explicit Simulation(asph_simulation* s, bool exports) : s_(s), exports_(exports) {}
    ~Simulation() { asph_simulation_destroy(s_); }
    Simulation(const Simulation&) = delete;
    Simulation& operator=(const Simulation&) = delete;

    void update(float deltaTime) {
        check(asph_simulation_update(s_, deltaTime), "asph_simulation_update");
        if (exports_) check(asph_simulation_export(s_), "asph_simulation_export");
    }
    void updateDomain(const asph_domain& domain, const StaticBoundaryDomain& boundaryDomain) {
        const auto& p = boundaryDomain.getParticles();
        check(asph_simulation_update_domain(s_, &domain, p.empty() ? nullptr : p.data(),
                                            static_cast<uint32_t>(p.size())),
              "asph_simulation_update_domain");
    }
    uint32_t getFluidParticlesCount() const {
        uint32_t n = 0;
        check(asph_simulation_fluid_count(s_, &n), "asph_simulation_fluid_count");
        return n;
    }
    uint32_t getBoundaryParticlesCount() const {
        uint32_t n = 0;
        check(asph_simulation_boundary_count(s_, &n), "asph_simulation_boundary_count");
        return n;
    }
    float calculateAverageNeighborCount() {
        float v = 0.0f;
        check(asph_simulation_average_neighbor_count(s_, &v), "asph_simulation_average_neighbor_count");
        return v;
    }
    DensityInfo getDensityInfo(float threshold) {
        DensityInfo d{};
        check(asph_simulation_density_info(s_, threshold, &d), "asph_simulation_density_info");
        return d;
    }
    void enableAdaptiveRefinement() {
        check(asph_simulation_enable_adaptive_refinement(s_), "asph_simulation_enable_adaptive_refinement");
    }
    // Particles copied to host memory (positions, velocities as vec4; densities, radii; ids), count of them.
    uint32_t readParticles(std::vector<vec4>& positions, std::vector<vec4>& velocities, std::vector<float>& densities,
                           std::vector<float>& radii, std::vector<uint32_t>& ids) const {
        const uint32_t n = getFluidParticlesCount();
        positions.resize(n);
        velocities.resize(n);
        densities.resize(n);
        radii.resize(n);
        ids.resize(n);
        check(asph_simulation_export_host(s_, positions.empty() ? nullptr : positions[0].data(),
                                          velocities.empty() ? nullptr : velocities[0].data(), densities.data(),
                                          radii.data(), ids.data(), n),
              "asph_simulation_export_host");
        return n;
    }
    // Enqueues a copy of the particles into caller-owned host arrays (pinned for the copy to overlap later steps)
    // and returns; the arrays hold them after waitForExport(). Returns the number of particles copied.
    uint32_t readParticlesAsync(vec4* positions, vec4* velocities, float* densities, float* radii, uint32_t* ids,
                                uint32_t capacity) {
        const uint32_t n = getFluidParticlesCount();
        check(asph_simulation_export_host_async(s_, positions ? positions->data() : nullptr,
                                                velocities ? velocities->data() : nullptr, densities, radii, ids,
                                                capacity),
              "asph_simulation_export_host_async");
        return n;
    }
    void waitForExport() { check(asph_simulation_export_wait(s_), "asph_simulation_export_wait"); }
    void stepAsync(float deltaTime) { check(asph_simulation_step_async(s_, deltaTime), "asph_simulation_step_async"); }
    asph_simulation* handle() const noexcept { return s_; }

private:
    asph_simulation* s_;
    bool exports_;
};

// createSimulation (Simulation.cuh:138-145): adaptive when the refinement parameters are given and enabled.
inline std::unique_ptr<Simulation> createSimulation(const Simulation::Parameters& parameters,
                                                    const std::vector<vec4>& positions,
                                                    const FluidParticlesDataImportedBuffer& fluidParticleMemory,
                                                    const BoundaryParticlesDataImportedBuffer& boundaryParticleMemory,
                                                    const StaticBoundaryDomain& boundaryDomain,
                                                    const std::optional<asph_refinement_parameters>& refinementParams,
                                                    uint32_t maxFluidParticleCapacity,
                                                    uint32_t maxBoundaryParticleCapacity) {
    auto h = [](const ImportedMemory* m) { return m ? m->handle() : nullptr; };
    const asph_fluid_buffers fb{h(fluidParticleMemory.positions), h(fluidParticleMemory.velocities),
                                h(fluidParticleMemory.densities), h(fluidParticleMemory.radii)};
    const asph_boundary_buffers bb{h(boundaryParticleMemory.positions), h(boundaryParticleMemory.radii),
                                   h(boundaryParticleMemory.colors)};
    const bool exports = fb.positions || fb.velocities || fb.densities || fb.radii;
    const bool walls = bb.positions || bb.radii || bb.colors;
    const auto& bp = boundaryDomain.getParticles();
    asph_simulation* s = nullptr;
    check(asph_simulation_create(&parameters, positions.empty() ? nullptr : positions[0].data(),
                                 static_cast<uint32_t>(positions.size()), exports ? &fb : nullptr,
                                 walls ? &bb : nullptr, bp.empty() ? nullptr : bp.data(),
                                 static_cast<uint32_t>(bp.size()), refinementParams ? &*refinementParams : nullptr,
                                 maxFluidParticleCapacity, maxBoundaryParticleCapacity, &s),
          "asph_simulation_create");
    return std::make_unique<Simulation>(s, exports);
}

}  // namespace asph

#endif  // ASPH_HPP
