// asph_device.cuh — device-side types and the canonical FP32 arithmetic of the particle pipeline.
//
// Compiled with -fmad=false: every fused multiply-add below is an explicit fmaf, every other product and
// sum is a separately rounded IEEE operation; division and square root are IEEE (-prec-div=true,
// -prec-sqrt=true). The CPU oracle performs the same operations, so results agree bit for bit.
//
// Formulas follow the reference: Wendland C2 kernel and derivative (cuda/src/algorithm/WendlandKernel.cuh:39-84),
// Tait equation of state with gamma = 5 (cuda/src/algorithm/Common.cuh:6-12). Departures in operation order:
// q = r * (1/h) with 1/h, coef/h^3 and dcoef/h^4 formed once per particle; the Tait term written as
// B*d*(5+d*(10+d*(10+d*(5+d)))), d = (rho-rho0)/rho0, which equals (rho/rho0)^5 - 1 without its cancellation.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace asph {

constexpr uint32_t kEmpty = 0xffffffffu;
constexpr uint32_t kNone = 0xffffffffu;
constexpr float kPi = 3.141592653589793f;

// Grid geometry: the reference grid (cell 4 h0, NeighborGrid.cu:108-121) and its 2x2x2 sub-cells.
struct GridDev {
    float dmin[3];
    float dmax[3];
    float scale[3];
    float cs[3];  // reference cell size
    float w[3];   // sub-cell size cs/2
    int32_t gs[3];
    int32_t sgs[3];
    uint32_t ncells;  // sub-cells
    uint32_t bits;    // Morton bits per axis
    int32_t periodic;
    float cull_margin;  // absolute widening of sub-cell boxes when culling (covers cell-assignment rounding)
};

// Fluid cell tables (sub-cell granularity) of the current step.
struct CellsDev {
    const uint32_t* start;
    const uint32_t* end;
    const float* hmax;       // max smoothing length of the members of each sub-cell
    const uint32_t* ex;      // [2] reference cells excluded by the reference's cell-boundary quirk
    const float* hmax_all;   // [1] max smoothing length over all particles
};

struct BoundaryDev {
    const float4* pos;  // x, y, z, psi (cell-sorted)
    const float* fric;
    const uint32_t* start;
    const uint32_t* end;
    const uint8_t* refflag;  // 1 where a reference cell holds boundary particles
    uint32_t ex0, ex1;
    uint32_t n;
};

struct PhysDev {
    float gravity[3];
    float c0, rho0, alpha, sigma, max_velocity, h0, r0, m0;
    float nu;
    float B;  // ((rho0*c0)*c0)/5
    int32_t morris;
    int32_t visc_on;
    int32_t sigma_on;
};

__device__ __forceinline__ float wcoef() { return 21.0f / (16.0f * kPi); }
__device__ __forceinline__ float dcoef() { return -5.0f * (21.0f / (16.0f * kPi)); }

__device__ __forceinline__ float dist2(float dx, float dy, float dz) { return fmaf(dz, dz, fmaf(dy, dy, dx * dx)); }

// W(r,h) with 1/h and coef/h^3 (WendlandKernel.cuh:39-52)
__device__ __forceinline__ float kernel_w(float r, float invh, float wc) {
    const float q = r * invh;
    if (q > 2.0f) return 0.0f;
    const float t = fmaf(-0.5f, q, 1.0f);
    const float t2 = t * t;
    return (wc * (t2 * t2)) * fmaf(2.0f, q, 1.0f);
}

// dW/dr(r,h) with 1/h and dcoef/h^4 (WendlandKernel.cuh:69-84)
__device__ __forceinline__ float kernel_dw(float r, float invh, float dwc) {
    const float q = r * invh;
    if (q > 2.0f) return 0.0f;
    const float t = fmaf(-0.5f, q, 1.0f);
    const float t3 = (t * t) * t;
    return (dwc * q) * t3;
}

// (1/h, coef/h^3, dcoef/h^4)
__device__ __forceinline__ void kernel_consts(float h, float& invh, float& wc, float& dwc) {
    const float h3 = (h * h) * h;
    invh = 1.0f / h;
    wc = wcoef() / h3;
    dwc = dcoef() / (h3 * h);
}

// p / rho^2 from the Tait equation (Common.cuh:6-12)
__device__ __forceinline__ float pressure_term(float rho, float rho0, float B) {
    const float d = (rho - rho0) / rho0;
    float u = 5.0f + d;
    u = fmaf(d, u, 10.0f);
    u = fmaf(d, u, 10.0f);
    u = fmaf(d, u, 5.0f);
    const float p = B * (d * u);
    return p / (rho * rho);
}

__device__ __forceinline__ uint32_t part1by2(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__device__ __forceinline__ uint32_t compact1by2(uint32_t x) {
    x &= 0x09249249u;
    x = (x ^ (x >> 2)) & 0x030c30c3u;
    x = (x ^ (x >> 4)) & 0x0300f00fu;
    x = (x ^ (x >> 8)) & 0xff0000ffu;
    x = (x ^ (x >> 16)) & 0x000003ffu;
    return x;
}

__device__ __forceinline__ uint32_t lin_of_key(const GridDev& g, uint32_t key) {
    const uint32_t x = compact1by2(key), y = compact1by2(key >> 1), z = compact1by2(key >> 2);
    return x + (uint32_t)g.sgs[0] * (y + (uint32_t)g.sgs[1] * z);
}

// calculateCellIndex + flattenCellIndex (NeighborGrid.cuh:166-177); sub-cell = floor(2f) of the same f.
__device__ __forceinline__ void cell_of(const GridDev& g, float px, float py, float pz, uint32_t& key,
                                        uint32_t& refkey) {
    const float p[3] = {px, py, pz};
    int32_t rc[3], sc[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float rel = p[a] - g.dmin[a];
        float cl = rel < 0.0f ? 0.0f : rel;
        cl = cl > g.scale[a] ? g.scale[a] : cl;
        const float f = cl / g.cs[a];
        int32_t c = (int32_t)f;
        if (c > g.gs[a] - 1) c = g.gs[a] - 1;
        int32_t s2 = (int32_t)(f * 2.0f);
        if (s2 > g.sgs[a] - 1) s2 = g.sgs[a] - 1;
        rc[a] = c;
        sc[a] = s2;
    }
    key = part1by2((uint32_t)sc[0]) | (part1by2((uint32_t)sc[1]) << 1) | (part1by2((uint32_t)sc[2]) << 2);
    refkey = (uint32_t)(rc[0] + g.gs[0] * (rc[1] + g.gs[1] * rc[2]));
}

__device__ __forceinline__ float clampf_(float x, float lo, float hi) {
    x = x < lo ? lo : x;
    return x > hi ? hi : x;
}

// Reference-cell range of the query box [x - R, x + R] on one axis (NeighborGrid.cuh:96-101), as the
// sub-cell range [2 lo, 2 hi + 1]. Returns false for an empty range.
__device__ __forceinline__ bool box_axis(const GridDev& g, int a, float p, float R, int32_t& slo, int32_t& shi) {
    const float rel = p - g.dmin[a];
    const float lof = clampf_((rel - R) / g.cs[a], -1.0e7f, 1.0e7f);
    const float hif = clampf_((rel + R) / g.cs[a], -1.0e7f, 1.0e7f);
    int32_t l, h;
    if (!g.periodic) {
        l = (int32_t)lof;
        h = (int32_t)hif;
        if (l < 0) l = 0;
        if (h > g.gs[a] - 1) h = g.gs[a] - 1;
    } else {
        l = (int32_t)floorf(lof);
        h = (int32_t)floorf(hif);
        if (h - l + 1 > g.gs[a]) h = l + g.gs[a] - 1;
    }
    slo = 2 * l;
    shi = 2 * h + 1;
    return l <= h;
}

// Narrows a sub-cell range to the sub-cells whose slab can hold a point within Rc of p (conservative; only
// ever skips sub-cells none of whose members can pass the distance test, so sums are unchanged).
__device__ __forceinline__ void trim_axis(const GridDev& g, int a, float p, float Rc, int32_t& slo, int32_t& shi) {
    const float rel = p - g.dmin[a];
    const float m = g.cull_margin;
    const int32_t lo2 = (int32_t)ceilf((rel - Rc - m) / g.w[a] - 1.0f);
    const int32_t hi2 = (int32_t)floorf((rel + Rc + m) / g.w[a]);
    slo = lo2 > slo ? lo2 : slo;
    shi = hi2 < shi ? hi2 : shi;
}

// Visits the candidate cells of a query in the canonical order (sub-cells z, y, x over the reference box),
// skipping the excluded reference cells and empty cells. With cull, sub-cells that cannot hold a member
// within 2*hmax(cell) (or within Rfix when Rfix > 0) of p are skipped as well.
// body(begin, end, sx, sy, sz) gets the member range [begin, end) and the periodic image shifts.
template <bool kCull, class Body>
__device__ __forceinline__ void for_each_cell(const GridDev& g, const uint32_t* __restrict__ start,
                                              const uint32_t* __restrict__ end, const float* __restrict__ hmax,
                                              uint32_t ex0, uint32_t ex1, float px, float py, float pz, float R,
                                              float Rtrim, float Rfix, Body&& body) {
    int32_t lo[3], hi[3];
    const float p[3] = {px, py, pz};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        ok &= box_axis(g, a, p[a], R, lo[a], hi[a]);
        if (kCull) trim_axis(g, a, p[a], Rtrim, lo[a], hi[a]);
    }
    if (!ok) return;
    for (int32_t sz = lo[2]; sz <= hi[2]; ++sz) {
        int32_t cz = sz;
        float shz = 0.0f;
        if (g.periodic) {
            if (cz < 0) { cz += g.sgs[2]; shz = -g.scale[2]; }
            else if (cz >= g.sgs[2]) { cz -= g.sgs[2]; shz = g.scale[2]; }
        }
        for (int32_t sy = lo[1]; sy <= hi[1]; ++sy) {
            int32_t cy = sy;
            float shy = 0.0f;
            if (g.periodic) {
                if (cy < 0) { cy += g.sgs[1]; shy = -g.scale[1]; }
                else if (cy >= g.sgs[1]) { cy -= g.sgs[1]; shy = g.scale[1]; }
            }
            for (int32_t sx = lo[0]; sx <= hi[0]; ++sx) {
                int32_t cx = sx;
                float shx = 0.0f;
                if (g.periodic) {
                    if (cx < 0) { cx += g.sgs[0]; shx = -g.scale[0]; }
                    else if (cx >= g.sgs[0]) { cx -= g.sgs[0]; shx = g.scale[0]; }
                    // a position more than one period outside the box (never after the first drift) has no cells
                    if (cx < 0 || cx >= g.sgs[0] || cy < 0 || cy >= g.sgs[1] || cz < 0 || cz >= g.sgs[2]) continue;
                } else {
                    const uint32_t rk = (uint32_t)((cx >> 1) + g.gs[0] * ((cy >> 1) + g.gs[1] * (cz >> 1)));
                    if (rk == ex0 || rk == ex1) continue;
                }
                const uint32_t lin = (uint32_t)cx + (uint32_t)g.sgs[0] * ((uint32_t)cy + (uint32_t)g.sgs[1] * (uint32_t)cz);
                const uint32_t b = __ldg(start + lin);
                if (b == kEmpty) continue;
                if (kCull) {
                    const float reach = Rfix > 0.0f ? Rfix : 2.0f * __ldg(hmax + lin);
                    // distance from p to the (widened) box of the sub-cell, in the unshifted frame of the cell
                    const float bx0 = g.dmin[0] + (float)cx * g.w[0] - g.cull_margin + shx;
                    const float by0 = g.dmin[1] + (float)cy * g.w[1] - g.cull_margin + shy;
                    const float bz0 = g.dmin[2] + (float)cz * g.w[2] - g.cull_margin + shz;
                    const float bw = 2.0f * g.cull_margin;
                    const float ddx = fmaxf(fmaxf(bx0 - px, px - (bx0 + g.w[0] + bw)), 0.0f);
                    const float ddy = fmaxf(fmaxf(by0 - py, py - (by0 + g.w[1] + bw)), 0.0f);
                    const float ddz = fmaxf(fmaxf(bz0 - pz, pz - (bz0 + g.w[2] + bw)), 0.0f);
                    const float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                    if (d2 > reach * reach * 1.0001f) continue;
                }
                body(b, __ldg(end + lin), shx, shy, shz);
            }
        }
    }
}

}  // namespace asph
