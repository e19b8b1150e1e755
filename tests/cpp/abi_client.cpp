// A C++ caller of the C ABI, the way the reference's app drives its simulation (app/App.cpp:144-251): generate the
// wall particles, create the simulation from host positions, step it, read the particles back.
//
// usage: abi_client <input> <output>
//   input : asph_parameters, float dt, uint32 steps, float wall spacing, uint32 n, n x float4 positions
//   output: uint32 n, n x float4 positions, n x float4 velocities, n x float densities, n x uint32 ids
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "asph.h"

namespace {

void check(asph_status s, const char* what) {
    if (s != ASPH_OK) throw std::runtime_error(std::string(what) + ": " + asph_last_error());
}

template <class T>
void read(std::FILE* f, T* p, size_t n) {
    if (std::fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short input");
}

template <class T>
void write(std::FILE* f, const T* p, size_t n) {
    if (std::fwrite(p, sizeof(T), n, f) != n) throw std::runtime_error("short output");
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
        return 2;
    }
    try {
        std::FILE* in = std::fopen(argv[1], "rb");
        if (!in) throw std::runtime_error("cannot open input");
        asph_parameters p{};
        float dt = 0.0f, spacing = 0.0f;
        uint32_t steps = 0, n = 0;
        read(in, &p, 1);
        read(in, &dt, 1);
        read(in, &steps, 1);
        read(in, &spacing, 1);
        read(in, &n, 1);
        std::vector<float> pos(4 * (size_t)n);
        read(in, pos.data(), pos.size());
        std::fclose(in);

        // StaticBoundaryDomain::generate: ask for the count, then fill
        uint32_t nb = 0;
        check(asph_boundary_generate(&p.domain, spacing, p.rest_density, p.base_smoothing_radius, nullptr, 0, &nb),
              "asph_boundary_generate");
        std::vector<asph_boundary_particle> walls(nb);
        check(asph_boundary_generate(&p.domain, spacing, p.rest_density, p.base_smoothing_radius, walls.data(), nb,
                                     &nb),
              "asph_boundary_generate");

        asph_simulation* sim = nullptr;
        check(asph_simulation_create(&p, pos.data(), n, nullptr, nullptr, walls.data(), nb, nullptr, n, nb, &sim),
              "asph_simulation_create");
        for (uint32_t k = 0; k < steps; k++) check(asph_simulation_update(sim, dt), "asph_simulation_update");

        uint32_t count = 0;
        check(asph_simulation_fluid_count(sim, &count), "asph_simulation_fluid_count");
        std::vector<float> opos(4 * (size_t)count), ovel(4 * (size_t)count), orho(count);
        std::vector<uint32_t> oid(count);
        check(asph_simulation_export_host(sim, opos.data(), ovel.data(), orho.data(), nullptr, oid.data(), count),
              "asph_simulation_export_host");
        asph_simulation_destroy(sim);

        std::FILE* out = std::fopen(argv[2], "wb");
        if (!out) throw std::runtime_error("cannot open output");
        write(out, &count, 1);
        write(out, opos.data(), opos.size());
        write(out, ovel.data(), ovel.size());
        write(out, orho.data(), orho.size());
        write(out, oid.data(), oid.size());
        std::fclose(out);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "abi_client: %s\n", e.what());
        return 1;
    }
    return 0;
}
