// The same run as abi_client.cpp through the C++ interface of asph.hpp, written the way the reference's app calls its
// simulation (app/App.cpp:144-251: StaticBoundaryDomain::generate, createSimulation, update per frame).
//
// usage: hpp_client <input> <output>   (formats as abi_client.cpp)
#include <cstdio>
#include <cstring>
#include <optional>
#include <stdexcept>
#include <vector>

#include "asph.hpp"

namespace {

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
        asph::Simulation::Parameters p{};
        float dt = 0.0f, spacing = 0.0f;
        uint32_t steps = 0, n = 0;
        read(in, &p, 1);
        read(in, &dt, 1);
        read(in, &steps, 1);
        read(in, &spacing, 1);
        read(in, &n, 1);
        std::vector<asph::vec4> positions(n);
        read(in, positions.empty() ? nullptr : positions[0].data(), 4 * (size_t)n);
        std::fclose(in);

        const auto boundary =
            asph::StaticBoundaryDomain::generate(p.domain, spacing, p.rest_density, p.base_smoothing_radius);
        auto simulation = asph::createSimulation(p, positions, {}, {}, boundary, std::nullopt, n,
                                                 boundary.getParticleCount());
        if (simulation->getBoundaryParticlesCount() != boundary.getParticleCount())
            throw std::runtime_error("boundary count");
        // the first half of the steps through update(), the rest enqueued with stepAsync() while the state after
        // the first half is copied out asynchronously (it must equal a synchronous read taken at the same point)
        const uint32_t half = steps / 2;
        for (uint32_t k = 0; k < half; k++) simulation->update(dt);
        std::vector<asph::vec4> mpos, mpos_async(simulation->getFluidParticlesCount());
        std::vector<asph::vec4> mvel;
        std::vector<float> mrho, mrad;
        std::vector<uint32_t> mid;
        simulation->readParticles(mpos, mvel, mrho, mrad, mid);
        simulation->readParticlesAsync(mpos_async.data(), nullptr, nullptr, nullptr, nullptr,
                                       static_cast<uint32_t>(mpos_async.size()));
        for (uint32_t k = half; k < steps; k++) simulation->stepAsync(dt);
        simulation->waitForExport();
        if (std::memcmp(mpos.data(), mpos_async.data(), mpos.size() * sizeof(asph::vec4)) != 0)
            throw std::runtime_error("asynchronous export differs from the synchronous one");

        std::vector<asph::vec4> opos, ovel;
        std::vector<float> orho, orad;
        std::vector<uint32_t> oid;
        const uint32_t count = simulation->readParticles(opos, ovel, orho, orad, oid);

        std::FILE* out = std::fopen(argv[2], "wb");
        if (!out) throw std::runtime_error("cannot open output");
        write(out, &count, 1);
        write(out, opos.empty() ? nullptr : opos[0].data(), 4 * (size_t)count);
        write(out, ovel.empty() ? nullptr : ovel[0].data(), 4 * (size_t)count);
        write(out, orho.data(), orho.size());
        write(out, oid.data(), oid.size());
        std::fclose(out);
    } catch (const asph::Error& e) {
        std::fprintf(stderr, "hpp_client: %s\n", e.what());
        return 1;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "hpp_client: %s\n", e.what());
        return 1;
    }
    return 0;
}
