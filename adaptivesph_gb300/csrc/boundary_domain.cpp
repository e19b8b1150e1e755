// boundary_domain.cpp — StaticBoundaryDomain::generate (cuda/include/cuda/simulation/physics/StaticBoundaryDomain.cuh:23-26,
// cuda/src/simulation/physics/StaticBoundaryDomain.cu:76-174) as host code behind asph_boundary_generate.
//
// Wall particles: six faces of the domain box widened by 0.05 m on every side, laid out with the reference's
// float loops (x += spacing), face order bottom, top, -x, +x, -z, +z. psi_b = rho0 / sum_{b'} W(|x_b - x_b'|, h)
// over walls with |d|^2 < (2h)^2, self included, W evaluated in the reference's own operation order
// (WendlandKernel.cuh:39-52). The reference finds neighbours with a nanoflann KD-tree and sums in tree order;
// here a uniform grid of cell 2h gives the same neighbour set and the sum runs in index order, so psi agrees
// to FP32 rounding. Built with -ffp-contract=off so the float loops match the reference's positions exactly.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/asph.h"

namespace {

float reference_wendland(float r, float h) {
    const float pi = 3.141592653589793f;
    const float q = r / h;
    if (q > 2.0f) return 0.0f;
    const float h3 = (h * h) * h;
    const float t = 1.0f - 0.5f * q;
    const float t4 = (t * t) * (t * t);
    return ((21.0f / (16.0f * pi)) / h3) * t4 * (2.0f * q + 1.0f);
}

void wall_positions(const asph_domain& d, float s, std::vector<float>& out) {
    float mn[3], mx[3];
    for (int a = 0; a < 3; a++) {
        mn[a] = d.min[a] - 0.05f;
        mx[a] = d.max[a] + 0.05f;
    }
    auto push = [&](float x, float y, float z) {
        out.push_back(x);
        out.push_back(y);
        out.push_back(z);
        out.push_back(0.0f);
    };
    for (float x = mn[0]; x < mx[0]; x += s)
        for (float z = mn[2]; z < mx[2]; z += s) push(x, mn[1], z);
    for (float x = mn[0]; x < mx[0]; x += s)
        for (float z = mn[2]; z < mx[2]; z += s) push(x, mx[1], z);
    for (float y = mn[1] + s; y < mx[1]; y += s)
        for (float z = mn[2]; z < mx[2]; z += s) push(mn[0], y, z);
    for (float y = mn[1] + s; y < mx[1]; y += s)
        for (float z = mn[2]; z < mx[2]; z += s) push(mx[0], y, z);
    for (float x = mn[0] + s; x < mx[0]; x += s)
        for (float y = mn[1] + s; y < mx[1]; y += s) push(x, y, mn[2]);
    for (float x = mn[0] + s; x < mx[0]; x += s)
        for (float y = mn[1] + s; y < mx[1]; y += s) push(x, y, mx[2]);
}

}  // namespace

extern "C" asph_status asph_boundary_generate(const asph_domain* bounds, float particle_spacing,
                                              float fluid_rest_density, float fluid_smoothing_radius,
                                              asph_boundary_particle* out, uint32_t capacity, uint32_t* count) {
    if (!bounds || !count) return ASPH_ERR_INVALID_ARGUMENT;
    if (!(particle_spacing > 0.0f) || !(fluid_smoothing_radius > 0.0f)) return ASPH_ERR_INVALID_ARGUMENT;
    for (int a = 0; a < 3; a++)
        if (!(bounds->max[a] > bounds->min[a])) return ASPH_ERR_INVALID_ARGUMENT;
    // bound the count before generating (each face holds about (extent / spacing + 2)^2 particles)
    {
        double total = 0.0;
        double e[3];
        for (int a = 0; a < 3; a++) e[a] = (bounds->max[a] - bounds->min[a] + 0.1) / particle_spacing + 2.0;
        total = 2.0 * (e[0] * e[2] + e[1] * e[2] + e[0] * e[1]);
        if (total > 4.0e9) return ASPH_ERR_CAPACITY;
    }
    std::vector<float> pos;
    wall_positions(*bounds, particle_spacing, pos);
    const size_t n = pos.size() / 4;
    *count = (uint32_t)n;
    if (!out) return ASPH_OK;
    if (n > capacity) return ASPH_ERR_CAPACITY;
    if (n == 0) return ASPH_OK;
    const float h = fluid_smoothing_radius;
    const float R = 2.0f * h;
    const float R2 = R * R;
    float lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = pos[a];
        hi[a] = pos[a];
    }
    for (size_t i = 0; i < n; i++)
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], pos[4 * i + a]);
            hi[a] = std::max(hi[a], pos[4 * i + a]);
        }
    int gd[3];
    for (int a = 0; a < 3; a++) gd[a] = (int)((hi[a] - lo[a]) / R) + 1;
    const size_t ncell = (size_t)gd[0] * gd[1] * gd[2];
    std::vector<uint32_t> head(ncell + 1, 0), list(n), cell(n);
    for (size_t i = 0; i < n; i++) {
        int c[3];
        for (int a = 0; a < 3; a++) c[a] = std::min(gd[a] - 1, (int)((pos[4 * i + a] - lo[a]) / R));
        cell[i] = (uint32_t)(c[0] + gd[0] * (c[1] + gd[1] * (size_t)c[2]));
        head[cell[i] + 1]++;
    }
    for (size_t c = 0; c < ncell; c++) head[c + 1] += head[c];
    {
        std::vector<uint32_t> fill(head.begin(), head.end() - 1);
        for (size_t i = 0; i < n; i++) list[fill[cell[i]]++] = (uint32_t)i;
    }
    auto work = [&](size_t i0, size_t i1) {
        std::vector<uint32_t> nb;
        for (size_t i = i0; i < i1; i++) {
            const uint32_t c = cell[i];
            const int cx = (int)(c % gd[0]), cy = (int)((c / gd[0]) % gd[1]), cz = (int)(c / ((size_t)gd[0] * gd[1]));
            nb.clear();
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const int x = cx + dx, y = cy + dy, z = cz + dz;
                        if (x < 0 || y < 0 || z < 0 || x >= gd[0] || y >= gd[1] || z >= gd[2]) continue;
                        const size_t cc = (size_t)x + gd[0] * ((size_t)y + gd[1] * (size_t)z);
                        for (uint32_t q = head[cc]; q < head[cc + 1]; q++) {
                            const uint32_t j = list[q];
                            const float ddx = pos[4 * i] - pos[4 * (size_t)j];
                            const float ddy = pos[4 * i + 1] - pos[4 * (size_t)j + 1];
                            const float ddz = pos[4 * i + 2] - pos[4 * (size_t)j + 2];
                            const float d2 = (ddx * ddx + ddy * ddy) + ddz * ddz;
                            if (d2 < R2) nb.push_back(j);
                        }
                    }
            std::sort(nb.begin(), nb.end());
            float sum = 0.0f;
            for (uint32_t j : nb) {
                const float ddx = pos[4 * i] - pos[4 * (size_t)j];
                const float ddy = pos[4 * i + 1] - pos[4 * (size_t)j + 1];
                const float ddz = pos[4 * i + 2] - pos[4 * (size_t)j + 2];
                const float d2 = (ddx * ddx + ddy * ddy) + ddz * ddz;
                sum += reference_wendland(std::sqrt(d2), h);
            }
            std::memcpy(out[i].position, &pos[4 * i], sizeof(float) * 4);
            out[i].psi = fluid_rest_density * (1.0f / sum);
        }
    };
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < 20000) nt = 1;
    std::vector<std::thread> th;
    const size_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++) {
        const size_t a = t * chunk, b = std::min(n, a + chunk);
        if (a < b) th.emplace_back(work, a, b);
    }
    for (auto& t : th) t.join();
    return ASPH_OK;
}
