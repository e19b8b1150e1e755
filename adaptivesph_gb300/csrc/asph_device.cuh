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
constexpr uint32_t kEligible = 0xfffffffeu;  // cand[] mark of a selected merge candidate before its search
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
    const float* hmax_ref;   // max smoothing length of the members of each reference cell (0: empty)
    const uint32_t* ex;      // [2] reference cells excluded by the reference's cell-boundary quirk
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

// Reference-cell range [lo, hi] of the query box [x - R, x + R] on one axis (NeighborGrid.cuh:96-101).
// Returns false for an empty range.
__device__ __forceinline__ bool box_axis(const GridDev& g, int a, float p, float R, int32_t& lo, int32_t& hi) {
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
    lo = l;
    hi = h;
    return l <= h;
}

// Number of reference cells in the query box [x - R, x + R].
__device__ __forceinline__ int box_cells(const GridDev& g, float4 p, float R) {
    int32_t lo, hi;
    int n = 1;
    const float pp[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (!box_axis(g, a, pp[a], R, lo, hi)) return 0;
        n *= (hi - lo + 1);
    }
    return n;
}

// Wraps a (possibly out-of-range) cell index of a periodic grid into [0, n) and returns the image offset.
__device__ __forceinline__ int32_t wrap_cell(int32_t c, int32_t n, float L, bool periodic, float& sh) {
    sh = 0.0f;
    if (periodic) {
        if (c < 0) {
            c += n;
            sh = -L;
        } else if (c >= n) {
            c -= n;
            sh = L;
        }
    }
    return c;
}

// Distance from p to the interval [lo, lo + w] widened by m on both sides.
__device__ __forceinline__ float gap1(float p, float lo, float w, float m) {
    return fmaxf(fmaxf((lo - m) - p, p - (lo + w + m)), 0.0f);
}

// Visits the candidate cells of a query in the canonical order: the reference cells of the box [x-R, x+R]
// (z, y, x order), skipping the cells excluded by the reference's cell-boundary quirk, and within each the
// 2x2x2 sub-cells (z, y, x order) that hold particles. With kCull, a reference cell or sub-cell that cannot
// hold a member within reach of p is skipped: reach = Rfix when Rfix > 0, else 2 * (max h of the cell). Culling
// never skips a member that passes a support test, so sums over the visited members are unchanged.
// body(begin, end, shx, shy, shz) gets the member range and the periodic image offsets.
template <bool kCull, class Body>
__device__ __forceinline__ void for_each_cell(const GridDev& g, const uint32_t* __restrict__ start,
                                              const uint32_t* __restrict__ end, const float* __restrict__ hmax,
                                              const float* __restrict__ hmax_ref, uint32_t ex0, uint32_t ex1,
                                              float px, float py, float pz, float R, float Rfix, Body&& body) {
    int32_t lo[3], hi[3];
    const float p[3] = {px, py, pz};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; a++) ok &= box_axis(g, a, p[a], R, lo[a], hi[a]);
    if (!ok) return;
    const bool periodic = g.periodic;
    const float m = g.cull_margin;
    for (int32_t rz = lo[2]; rz <= hi[2]; ++rz) {
        for (int32_t ry = lo[1]; ry <= hi[1]; ++ry) {
            for (int32_t rx = lo[0]; rx <= hi[0]; ++rx) {
                float shz, shy, shx;
                const int32_t cz = wrap_cell(rz, g.gs[2], g.scale[2], periodic, shz);
                if (cz < 0 || cz >= g.gs[2]) continue;
                const int32_t cy = wrap_cell(ry, g.gs[1], g.scale[1], periodic, shy);
                if (cy < 0 || cy >= g.gs[1]) continue;
                const int32_t cx = wrap_cell(rx, g.gs[0], g.scale[0], periodic, shx);
                if (cx < 0 || cx >= g.gs[0]) continue;
                const uint32_t rk = (uint32_t)cx + (uint32_t)g.gs[0] * ((uint32_t)cy + (uint32_t)g.gs[1] * (uint32_t)cz);
                if (!periodic && (rk == ex0 || rk == ex1)) continue;
                // sub-cell ranges of this reference cell, narrowed to the slabs within reach
                int32_t s0[3] = {2 * cx, 2 * cy, 2 * cz}, s1[3] = {2 * cx + 1, 2 * cy + 1, 2 * cz + 1};
                if (kCull) {
                    const float hr = __ldg(hmax_ref + rk);
                    if (hr <= 0.0f) continue;  // no particles in this reference cell
                    const float reach = (Rfix > 0.0f ? Rfix : 2.0f * hr) * 1.00005f;
                    const float sh[3] = {shx, shy, shz};
                    const int32_t c3[3] = {cx, cy, cz};
                    float d2 = 0.0f;
                    bool any = true;
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        const float base = g.dmin[a] + (float)c3[a] * g.cs[a] + sh[a];
                        const float d = gap1(p[a], base, g.cs[a], m);
                        d2 += d * d;
                        const bool k0 = gap1(p[a], base, g.w[a], m) <= reach;
                        const bool k1 = gap1(p[a], base + g.w[a], g.w[a], m) <= reach;
                        s0[a] = k0 ? 2 * c3[a] : 2 * c3[a] + 1;
                        s1[a] = k1 ? 2 * c3[a] + 1 : 2 * c3[a];
                        any &= (k0 || k1);
                    }
                    if (!any || d2 > reach * reach) continue;
                }
                for (int32_t sz = s0[2]; sz <= s1[2]; ++sz)
                    for (int32_t sy = s0[1]; sy <= s1[1]; ++sy)
                        for (int32_t sx = s0[0]; sx <= s1[0]; ++sx) {
                            const uint32_t lin =
                                (uint32_t)sx + (uint32_t)g.sgs[0] * ((uint32_t)sy + (uint32_t)g.sgs[1] * (uint32_t)sz);
                            const uint32_t b = __ldg(start + lin);
                            if (b == kEmpty) continue;
                            if (kCull) {
                                const float reach = (Rfix > 0.0f ? Rfix : 2.0f * __ldg(hmax + lin)) * 1.00005f;
                                const float dx = gap1(px, g.dmin[0] + (float)sx * g.w[0] + shx, g.w[0], m);
                                const float dy = gap1(py, g.dmin[1] + (float)sy * g.w[1] + shy, g.w[1], m);
                                const float dz = gap1(pz, g.dmin[2] + (float)sz * g.w[2] + shz, g.w[2], m);
                                if (dx * dx + dy * dy + dz * dz > reach * reach) continue;
                            }
                            body(b, __ldg(end + lin), shx, shy, shz);
                        }
            }
        }
    }
}

// One query walked by a whole warp: the sub-cells of the box [x-R, x+R] are numbered in the canonical order,
// t = 8 * (index of the reference cell in z, y, x order within the box) + (sub-cell z, y, x bits), and lane l
// visits those with t mod 32 == l, in increasing t. Excluded, empty and culled sub-cells are skipped (culling as in
// for_each_cell<true>: reach = Rfix when Rfix > 0, else 2 * max h of the sub-cell); so the 32 lanes walk a large
// box in 1/32 of the sequential walk, and each lane's visiting order is fixed by the box alone.
// The walk is two-level: 32 reference cells at a time are tested against their max h (one cell per lane), and
// only the surviving cells are opened. Lane l owns sub-cell (l mod 8) of the cells whose index in the box is
// congruent to l / 8 modulo 4, so the four groups of 8 lanes open their own survivors side by side, each in
// increasing cell order. The query (px, py, pz, R) must be the same on every lane.
template <class Body>
__device__ __forceinline__ void for_each_subcell_lane(const GridDev& g, const uint32_t* __restrict__ start,
                                                      const uint32_t* __restrict__ end,
                                                      const float* __restrict__ hmax,
                                                      const float* __restrict__ hmax_ref, uint32_t ex0, uint32_t ex1,
                                                      float px, float py, float pz, float R, float Rfix, int lane,
                                                      Body&& body, uint32_t wi = 0, uint32_t nw = 1) {
    int32_t lo[3], hi[3];
    const float p[3] = {px, py, pz};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; a++) ok &= box_axis(g, a, p[a], R, lo[a], hi[a]);
    if (!ok) return;
    const uint32_t nx = (uint32_t)(hi[0] - lo[0] + 1), ny = (uint32_t)(hi[1] - lo[1] + 1);
    const uint32_t nz = (uint32_t)(hi[2] - lo[2] + 1);
    const uint32_t ncell = nx * ny * nz;
    const bool periodic = g.periodic;
    const float m = g.cull_margin;
    const uint32_t grp = (uint32_t)lane >> 3, q = (uint32_t)lane & 7u;
    const int32_t qx = (int32_t)(q & 1u), qy = (int32_t)((q >> 1) & 1u), qz = (int32_t)(q >> 2);
    // with nw warps over one box (wi this warp's index), warp wi takes the reference cells whose index modulo 4 nw is
    // in [4 wi, 4 wi + 4), 32 of them per round; with one warp that is cells base + lane, base = 0, 32, 64, ...
    const uint32_t G = 4u * nw;
    for (uint32_t j0 = 0; G * j0 + 4u * wi < ncell; j0 += 8u) {
        // level 1: one reference cell per lane
        const uint32_t cell = G * (j0 + ((uint32_t)lane >> 2)) + 4u * wi + ((uint32_t)lane & 3u);
        float shx = 0.0f, shy = 0.0f, shz = 0.0f;
        int32_t cx = 0, cy = 0, cz = 0;
        bool live = false;
        if (cell < ncell) {
            const uint32_t cxy = cell % (nx * ny);
            cz = wrap_cell(lo[2] + (int32_t)(cell / (nx * ny)), g.gs[2], g.scale[2], periodic, shz);
            cy = wrap_cell(lo[1] + (int32_t)(cxy / nx), g.gs[1], g.scale[1], periodic, shy);
            cx = wrap_cell(lo[0] + (int32_t)(cxy % nx), g.gs[0], g.scale[0], periodic, shx);
            if (cz >= 0 && cz < g.gs[2] && cy >= 0 && cy < g.gs[1] && cx >= 0 && cx < g.gs[0]) {
                const uint32_t rk =
                    (uint32_t)cx + (uint32_t)g.gs[0] * ((uint32_t)cy + (uint32_t)g.gs[1] * (uint32_t)cz);
                const float hr = __ldg(hmax_ref + rk);
                if (hr > 0.0f && (periodic || (rk != ex0 && rk != ex1))) {
                    const float reach = (Rfix > 0.0f ? Rfix : 2.0f * hr) * 1.00005f;
                    const float dx = gap1(px, g.dmin[0] + (float)cx * g.cs[0] + shx, g.cs[0], m);
                    const float dy = gap1(py, g.dmin[1] + (float)cy * g.cs[1] + shy, g.cs[1], m);
                    const float dz = gap1(pz, g.dmin[2] + (float)cz * g.cs[2] + shz, g.cs[2], m);
                    live = dx * dx + dy * dy + dz * dz <= reach * reach;
                }
            }
        }
        // level 2: each group of 8 lanes opens its survivors (cells congruent to the group modulo 4) in order
        uint32_t mine = __ballot_sync(0xffffffffu, live) & (0x11111111u << grp);
        while (__any_sync(0xffffffffu, mine != 0u)) {
            const bool has = mine != 0u;
            const int src = has ? __ffs(mine) - 1 : lane;
            mine &= mine - 1u;
            const int32_t ox = __shfl_sync(0xffffffffu, cx, src), oy = __shfl_sync(0xffffffffu, cy, src),
                          oz = __shfl_sync(0xffffffffu, cz, src);
            const float sx_ = __shfl_sync(0xffffffffu, shx, src), sy_ = __shfl_sync(0xffffffffu, shy, src),
                        sz_ = __shfl_sync(0xffffffffu, shz, src);
            if (!has) continue;  // this group has no survivor left
            const int32_t sx = 2 * ox + qx, sy = 2 * oy + qy, sz = 2 * oz + qz;
            const uint32_t lin =
                (uint32_t)sx + (uint32_t)g.sgs[0] * ((uint32_t)sy + (uint32_t)g.sgs[1] * (uint32_t)sz);
            const uint32_t b = __ldg(start + lin);
            if (b == kEmpty) continue;
            const float hs = __ldg(hmax + lin);
            const float reach = (Rfix > 0.0f ? Rfix : 2.0f * hs) * 1.00005f;
            const float dx = gap1(px, g.dmin[0] + (float)sx * g.w[0] + sx_, g.w[0], m);
            const float dy = gap1(py, g.dmin[1] + (float)sy * g.w[1] + sy_, g.w[1], m);
            const float dz = gap1(pz, g.dmin[2] + (float)sz * g.w[2] + sz_, g.w[2], m);
            if (dx * dx + dy * dy + dz * dz > reach * reach) continue;
            body(b, __ldg(end + lin), sx_, sy_, sz_);
        }
    }
}

// Boundary cells of the query box [x-R, x+R] in the canonical order (reference cells z, y, x; their sub-cells z, y, x),
// skipping excluded reference cells, reference cells without boundary particles and cells or sub-cells farther than
// R from p (R is the support radius of the boundary sums, so a skipped sub-cell holds no member with r <= R).
// body(begin, end, shx, shy, shz) gets each remaining sub-cell's member range.
// kLanes == 1: one lane walks alone. kLanes == 32: the whole warp walks one query (the same on every lane) and
// calls body warp-uniformly; 32 reference cells are tested at a time, one per lane.
template <int kLanes, class Body>
__device__ __forceinline__ void for_each_boundary_cell(const GridDev& g, const BoundaryDev& b, float px, float py,
                                                       float pz, float R, int lane, Body&& body) {
    if (b.n == 0) return;
    int32_t lo[3], hi[3];
    const float p[3] = {px, py, pz};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; a++) ok &= box_axis(g, a, p[a], R, lo[a], hi[a]);
    if (!ok) return;
    const bool periodic = g.periodic;
    const float m = g.cull_margin;
    const float reach = R * 1.00005f;
    const float reach2 = reach * reach;
    // reference cell (rx, ry, rz) of the box: wrapped coordinates, image offsets, and whether it can contribute
    auto ref_live = [&](int32_t rx, int32_t ry, int32_t rz, int32_t& cx, int32_t& cy, int32_t& cz, float& shx,
                        float& shy, float& shz) -> bool {
        cz = wrap_cell(rz, g.gs[2], g.scale[2], periodic, shz);
        cy = wrap_cell(ry, g.gs[1], g.scale[1], periodic, shy);
        cx = wrap_cell(rx, g.gs[0], g.scale[0], periodic, shx);
        if (cz < 0 || cz >= g.gs[2] || cy < 0 || cy >= g.gs[1] || cx < 0 || cx >= g.gs[0]) return false;
        const uint32_t rk = (uint32_t)cx + (uint32_t)g.gs[0] * ((uint32_t)cy + (uint32_t)g.gs[1] * (uint32_t)cz);
        if (!periodic && (rk == b.ex0 || rk == b.ex1)) return false;
        if (!__ldg(b.refflag + rk)) return false;
        const float dx = gap1(px, g.dmin[0] + (float)cx * g.cs[0] + shx, g.cs[0], m);
        const float dy = gap1(py, g.dmin[1] + (float)cy * g.cs[1] + shy, g.cs[1], m);
        const float dz = gap1(pz, g.dmin[2] + (float)cz * g.cs[2] + shz, g.cs[2], m);
        return dx * dx + dy * dy + dz * dz <= reach2;
    };
    // sub-cell (sx, sy, sz): its member range when it is non-empty and within reach
    auto sub_live = [&](int32_t sx, int32_t sy, int32_t sz, float shx, float shy, float shz, uint32_t& kb,
                        uint32_t& ke) -> bool {
        const uint32_t lin = (uint32_t)sx + (uint32_t)g.sgs[0] * ((uint32_t)sy + (uint32_t)g.sgs[1] * (uint32_t)sz);
        kb = __ldg(b.start + lin);
        if (kb == kEmpty) return false;
        const float dx = gap1(px, g.dmin[0] + (float)sx * g.w[0] + shx, g.w[0], m);
        const float dy = gap1(py, g.dmin[1] + (float)sy * g.w[1] + shy, g.w[1], m);
        const float dz = gap1(pz, g.dmin[2] + (float)sz * g.w[2] + shz, g.w[2], m);
        if (dx * dx + dy * dy + dz * dz > reach2) return false;
        ke = __ldg(b.end + lin);
        return true;
    };
    if (kLanes == 1) {
        for (int32_t rz = lo[2]; rz <= hi[2]; ++rz)
            for (int32_t ry = lo[1]; ry <= hi[1]; ++ry)
                for (int32_t rx = lo[0]; rx <= hi[0]; ++rx) {
                    int32_t cx, cy, cz;
                    float shx, shy, shz;
                    if (!ref_live(rx, ry, rz, cx, cy, cz, shx, shy, shz)) continue;
#pragma unroll 1
                    for (int q = 0; q < 8; ++q) {
                        uint32_t kb, ke;
                        if (sub_live(2 * cx + (q & 1), 2 * cy + ((q >> 1) & 1), 2 * cz + (q >> 2), shx, shy, shz, kb,
                                     ke))
                            body(kb, ke, shx, shy, shz);
                    }
                }
        return;
    }
    const uint32_t nx = (uint32_t)(hi[0] - lo[0] + 1), ny = (uint32_t)(hi[1] - lo[1] + 1);
    const uint32_t ncell = nx * ny * (uint32_t)(hi[2] - lo[2] + 1);
    for (uint32_t base = 0; base < ncell; base += 32u) {
        const uint32_t cell = base + (uint32_t)lane;
        int32_t cx = 0, cy = 0, cz = 0;
        float shx = 0.0f, shy = 0.0f, shz = 0.0f;
        bool live = false;
        if (cell < ncell) {
            const uint32_t cxy = cell % (nx * ny);
            live = ref_live(lo[0] + (int32_t)(cxy % nx), lo[1] + (int32_t)(cxy / nx), lo[2] + (int32_t)(cell / (nx * ny)),
                            cx, cy, cz, shx, shy, shz);
        }
        uint32_t cells = __ballot_sync(0xffffffffu, live);
        while (cells != 0u) {
            const int src = __ffs(cells) - 1;
            cells &= cells - 1u;
            const int32_t ox = __shfl_sync(0xffffffffu, cx, src), oy = __shfl_sync(0xffffffffu, cy, src),
                          oz = __shfl_sync(0xffffffffu, cz, src);
            const float sx_ = __shfl_sync(0xffffffffu, shx, src), sy_ = __shfl_sync(0xffffffffu, shy, src),
                        sz_ = __shfl_sync(0xffffffffu, shz, src);
            // lanes 0-7 look at the eight sub-cells, then the warp visits the live ones in order
            uint32_t kb = 0, ke = 0;
            const bool sl = lane < 8 && sub_live(2 * ox + (lane & 1), 2 * oy + ((lane >> 1) & 1), 2 * oz + (lane >> 2),
                                                 sx_, sy_, sz_, kb, ke);
            uint32_t subs = __ballot_sync(0xffffffffu, sl);
            while (subs != 0u) {
                const int q = __ffs(subs) - 1;
                subs &= subs - 1u;
                body(__shfl_sync(0xffffffffu, kb, q), __shfl_sync(0xffffffffu, ke, q), sx_, sy_, sz_);
            }
        }
    }
}

// Warp-cooperative form of for_each_cell<true> for the 32 particles of a warp (one per lane; `active` lanes only).
// The warp walks the union of the lanes' boxes in the canonical order (reference cells z, y, x; their sub-cells
// z, y, x) and calls body(begin, end, shx, shy, shz, need) warp-uniformly for every sub-cell that some lane needs;
// `need` tells the calling lane whether the sub-cell is one of its own candidate cells that survived its culling.
// Restricted to one lane, the visited sequence is exactly that lane's for_each_cell<true> sequence, so per-lane
// sums keep their order; lanes share every candidate load. Returns false (having visited nothing) when the union
// spans more than max_union reference cells; the caller then falls back to for_each_cell per lane.
template <class Body>
__device__ __forceinline__ bool for_each_cell_warp(const GridDev& g, const uint32_t* __restrict__ start,
                                                   const uint32_t* __restrict__ end, const float* __restrict__ hmax,
                                                   const float* __restrict__ hmax_ref, uint32_t ex0, uint32_t ex1,
                                                   bool active, float px, float py, float pz, float R,
                                                   int32_t max_union, Body&& body) {
    int32_t lo[3], hi[3];
    const float p[3] = {px, py, pz};
    bool ok = active;
#pragma unroll
    for (int a = 0; a < 3; a++) ok &= box_axis(g, a, p[a], R, lo[a], hi[a]);
    int32_t ulo[3], uhi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        ulo[a] = __reduce_min_sync(0xffffffffu, ok ? lo[a] : 0x7fffffff);
        uhi[a] = __reduce_max_sync(0xffffffffu, ok ? hi[a] : (int32_t)0x80000000);
    }
    if (!__any_sync(0xffffffffu, ok)) return true;
    const int64_t span = (int64_t)(uhi[0] - ulo[0] + 1) * (uhi[1] - ulo[1] + 1) * (uhi[2] - ulo[2] + 1);
    if (span > max_union || span > 64) return false;
    const bool periodic = g.periodic;
    const float m = g.cull_margin;
    const int lane = (int)(threadIdx.x & 31u);
    // The union's reference cells are numbered in walk order, t = ((rz - ulo) * ny + (ry - ulo)) * nx + (rx - ulo);
    // lane l fetches the max h of cells l and l + 32 up front (0 outside the grid or for an excluded cell), and the
    // walk takes each cell's from a shuffle instead of a load it would wait for.
    const int32_t nx = uhi[0] - ulo[0] + 1, ny = uhi[1] - ulo[1] + 1;
    auto ref_hmax = [&](int32_t t) -> float {
        if (t >= (int32_t)span) return 0.0f;
        const int32_t rx = ulo[0] + t % nx, ry = ulo[1] + (t / nx) % ny, rz = ulo[2] + t / (nx * ny);
        float sh;
        const int32_t cz = wrap_cell(rz, g.gs[2], g.scale[2], periodic, sh);
        const int32_t cy = wrap_cell(ry, g.gs[1], g.scale[1], periodic, sh);
        const int32_t cx = wrap_cell(rx, g.gs[0], g.scale[0], periodic, sh);
        if (cz < 0 || cz >= g.gs[2] || cy < 0 || cy >= g.gs[1] || cx < 0 || cx >= g.gs[0]) return 0.0f;
        const uint32_t rk = (uint32_t)cx + (uint32_t)g.gs[0] * ((uint32_t)cy + (uint32_t)g.gs[1] * (uint32_t)cz);
        if (!periodic && (rk == ex0 || rk == ex1)) return 0.0f;
        return __ldg(hmax_ref + rk);
    };
    const float hr_lo = ref_hmax(lane), hr_hi = ref_hmax(lane + 32);
    for (int32_t rz = ulo[2]; rz <= uhi[2]; ++rz) {
        for (int32_t ry = ulo[1]; ry <= uhi[1]; ++ry) {
            for (int32_t rx = ulo[0]; rx <= uhi[0]; ++rx) {
                const int32_t t = ((rz - ulo[2]) * ny + (ry - ulo[1])) * nx + (rx - ulo[0]);
                const float hr = __shfl_sync(0xffffffffu, t < 32 ? hr_lo : hr_hi, t & 31);
                if (hr <= 0.0f) continue;  // empty, outside the grid or excluded
                float shz, shy, shx;
                const int32_t cz = wrap_cell(rz, g.gs[2], g.scale[2], periodic, shz);
                const int32_t cy = wrap_cell(ry, g.gs[1], g.scale[1], periodic, shy);
                const int32_t cx = wrap_cell(rx, g.gs[0], g.scale[0], periodic, shx);
                // the eight sub-cells' member ranges and max h, fetched by lanes 0-7 at once, issued before the
                // reach tests below so that their latency overlaps them (fetched for every octant: the tables
                // hold every sub-cell, and only the non-empty ones are used)
                uint32_t sb = kEmpty, se = 0u;
                float shm = 0.0f;
                if (lane < 8) {
                    const int32_t sx = 2 * cx + (lane & 1), sy = 2 * cy + ((lane >> 1) & 1), sz = 2 * cz + (lane >> 2);
                    const uint32_t lin =
                        (uint32_t)sx + (uint32_t)g.sgs[0] * ((uint32_t)sy + (uint32_t)g.sgs[1] * (uint32_t)sz);
                    sb = __ldg(start + lin);
                    se = __ldg(end + lin);
                    shm = __ldg(hmax + lin);
                }
                bool need = ok && rx >= lo[0] && rx <= hi[0] && ry >= lo[1] && ry <= hi[1] && rz >= lo[2] &&
                            rz <= hi[2];
                const float reach = 2.0f * hr * 1.00005f;
                const float sh[3] = {shx, shy, shz};
                const int32_t c3[3] = {cx, cy, cz};
                // squared distances to the lower and upper sub-cell slab on each axis
                float q0[3], q1[3];
                float d2 = 0.0f;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const float base = g.dmin[a] + (float)c3[a] * g.cs[a] + sh[a];
                    const float d = gap1(p[a], base, g.cs[a], m);
                    d2 += d * d;
                    const float e0 = gap1(p[a], base, g.w[a], m), e1 = gap1(p[a], base + g.w[a], g.w[a], m);
                    q0[a] = e0 * e0;
                    q1[a] = e1 * e1;
                }
                need &= d2 <= reach * reach;
                if (!__any_sync(0xffffffffu, need)) continue;
                uint32_t live = __ballot_sync(0xffffffffu, sb != kEmpty) & 0xffu;
                // the sub-cells some lane may need, tested against the reference cell's max h (at least each
                // sub-cell's, so no sub-cell a lane needs is dropped; the exact test below stays as it was): the
                // loop then visits only those instead of every non-empty one. e2 of octant q is summed as below,
                // x + y first, so the two tests see the same value.
                uint32_t may = 0u;
                if (need) {
                    const float rr = reach * reach;
                    const float s00 = q0[0] + q0[1], s10 = q1[0] + q0[1], s01 = q0[0] + q1[1], s11 = q1[0] + q1[1];
                    may = (s00 + q0[2] <= rr ? 0x01u : 0u) | (s10 + q0[2] <= rr ? 0x02u : 0u) |
                          (s01 + q0[2] <= rr ? 0x04u : 0u) | (s11 + q0[2] <= rr ? 0x08u : 0u) |
                          (s00 + q1[2] <= rr ? 0x10u : 0u) | (s10 + q1[2] <= rr ? 0x20u : 0u) |
                          (s01 + q1[2] <= rr ? 0x40u : 0u) | (s11 + q1[2] <= rr ? 0x80u : 0u);
                }
                live &= __reduce_or_sync(0xffffffffu, may);
                while (live != 0u) {
                    const int q = __ffs(live) - 1;
                    live &= live - 1u;
                    const uint32_t b = __shfl_sync(0xffffffffu, sb, q), e = __shfl_sync(0xffffffffu, se, q);
                    const float hs = __shfl_sync(0xffffffffu, shm, q);
                    bool ns = need;
                    if (ns) {
                        const float rs = 2.0f * hs * 1.00005f;
                        const float e2 = ((q & 1) ? q1[0] : q0[0]) + ((q & 2) ? q1[1] : q0[1]) + ((q & 4) ? q1[2] : q0[2]);
                        ns = e2 <= rs * rs;
                    }
                    if (!__any_sync(0xffffffffu, ns)) continue;
                    body(b, e, shx, shy, shz, ns);
                }
            }
        }
    }
    return true;
}

}  // namespace asph
