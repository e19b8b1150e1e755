// neighbor_kernels.cu — the neighbour passes of a step: density (+ neighbour lists) and forces.
//
// computeDensities / computeBoundaryDensityContribution (cuda/src/algorithm/Algorithm.cu:17-54,
// cuda/src/algorithm/BoundaryAlgorithm.cu:15-51) and the acceleration kernels (Algorithm.cu:56-232,
// BoundaryAlgorithm.cu:53-162) of SphSimulation::update (cuda/src/simulation/SphSimulation.cu:101-120).
//
// Ordinary particles: one thread per particle. In the density pass the 32 particles of a warp (neighbours in the
// cell order) walk the union of their candidate cells together in the canonical order, each lane testing every
// candidate of its own cells (shared loads, no divergent loop control) and recording its accepted neighbours (self
// included) in its row of the neighbour list. A row entry covers one block of up to 32 consecutive members of a
// sub-cell: (first member | periodic image code, 32-bit acceptance mask), 8 bytes, written only for blocks holding
// an accepted neighbour. Entries are written in 16-byte pairs (an even entry waits in registers for its partner).
// Each lane then sums its density over its row, and the force pass sums over the same row: the masks expanded in
// member order give the accepted neighbours in the canonical order, two per loop iteration in packed FP32x2. The
// boundary density records the accepted wall blocks after the fluid entries in the same form, and the force pass
// forms the wall terms from them.
// Heavy particles (query box of more than 27 reference cells: smoothing lengths grown by merging) and particles
// with more entries than a row holds: one warp per particle; the box's sub-cells are dealt to the lanes by their
// canonical index (for_each_subcell_lane), each lane sums its sub-cells' members in order, and the lane sums are
// combined by a fixed butterfly. They are queued for separate warp kernels, so a few large boxes do not stall
// whole blocks.
#include <utility>

#include "asph_device.cuh"
#include "asph_kernels.cuh"

namespace asph {

namespace {

constexpr uint32_t kIdxBits = 27;
constexpr uint32_t kIdxMask = (1u << kIdxBits) - 1u;
constexpr int32_t kMaxUnion = 40;  // a warp walks its lanes' boxes together when their union is at most this big

// Periodic image of a listed neighbour: the index keeps 27 bits, the cell's image offset (-1, 0, +1 per axis)
// is packed into the top 5 bits.
__device__ __forceinline__ uint32_t shift_code(float shx, float shy, float shz) {
    const int cx = shx < 0.0f ? 0 : (shx > 0.0f ? 2 : 1);
    const int cy = shy < 0.0f ? 0 : (shy > 0.0f ? 2 : 1);
    const int cz = shz < 0.0f ? 0 : (shz > 0.0f ? 2 : 1);
    return (uint32_t)(cx + 3 * cy + 9 * cz);
}

__device__ __forceinline__ void decode_entry(const GridDev& g, uint32_t e, uint32_t& j, float& shx, float& shy,
                                             float& shz) {
    if (!g.periodic) {
        j = e;
        shx = shy = shz = 0.0f;
        return;
    }
    j = e & kIdxMask;
    const uint32_t code = e >> kIdxBits;
    const int cx = (int)(code % 3u), cy = (int)((code / 3u) % 3u), cz = (int)(code / 9u);
    shx = cx == 0 ? -g.scale[0] : (cx == 2 ? g.scale[0] : 0.0f);
    shy = cy == 0 ? -g.scale[1] : (cy == 2 ? g.scale[1] : 0.0f);
    shz = cz == 0 ? -g.scale[2] : (cz == 2 ? g.scale[2] : 0.0f);
}

// A row entry: first member (and periodic image offset) and acceptance mask of a block.
__device__ __forceinline__ void row_entry(const GridDev& g, uint2 en, uint32_t& first, uint32_t& mask, float& shx,
                                          float& shy, float& shz) {
    decode_entry(g, en.x, first, shx, shy, shz);
    mask = en.y;
}

__device__ __forceinline__ float warp_sum_butterfly(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// The support test r^2 <= (2 h_j)^2 of neighbour position pj (periodic image offset applied) for p.
__device__ __forceinline__ bool supported(const GridDev& g, float4 p, float4 pj, float shx, float shy, float shz) {
    const bool periodic = g.periodic;
    const float xj = periodic ? pj.x + shx : pj.x;
    const float yj = periodic ? pj.y + shy : pj.y;
    const float zj = periodic ? pj.z + shz : pj.z;
    const float dx = xj - p.x, dy = yj - p.y, dz = zj - p.z;
    const float twoh = pj.w + pj.w;
    return dist2(dx, dy, dz) <= twoh * twoh;
}

// Fluid density term of neighbour j (Algorithm.cu:29-51); false when j fails r^2 <= (2 h_j)^2.
__device__ __forceinline__ bool density_term(const StepArgs& a, float4 pi, uint32_t j, float shx, float shy,
                                             float shz, float& rho) {
    const float4 pj = __ldg(a.ph + j);
    const bool periodic = a.grid.periodic;
    const float xj = periodic ? pj.x + shx : pj.x;
    const float yj = periodic ? pj.y + shy : pj.y;
    const float zj = periodic ? pj.z + shz : pj.z;
    const float dx = xj - pi.x, dy = yj - pi.y, dz = zj - pi.z;
    const float r2 = dist2(dx, dy, dz);
    const float twoh = pj.w + pj.w;
    if (r2 > twoh * twoh) return false;
    const float4 kj = __ldg(a.kc + j);
    const float w = kernel_w(sqrtf(r2), kj.x, kj.y);
    rho = fmaf(kj.w, w, rho);
    return true;
}

// density_term of a neighbour from the particle's row (accepted by the scan's support test on the same operands):
// the position from pq, as in density_pair<..., true>.
__device__ __forceinline__ void density_term_accepted(const StepArgs& a, float4 pi, uint32_t j, float shx, float shy,
                                                      float shz, float& rho) {
    const float4 pj = __ldg(a.pq + j);
    const bool periodic = a.grid.periodic;
    const float xj = periodic ? pj.x + shx : pj.x;
    const float yj = periodic ? pj.y + shy : pj.y;
    const float zj = periodic ? pj.z + shz : pj.z;
    const float dx = xj - pi.x, dy = yj - pi.y, dz = zj - pi.z;
    const float r2 = dist2(dx, dy, dz);
    const float4 kj = __ldg(a.kc + j);
    const float w = kernel_w(sqrtf(r2), kj.x, kj.y);
    rho = fmaf(kj.w, w, rho);
}

// density_term for two neighbours, in packed FP32x2 arithmetic (each half rounds as the scalar operation), added in
// order: j1 then j2. kAccepted: both are members of the particle's row, accepted by the same support test (same
// operands, same operations) in the scan, so the test is not repeated.
// With kAccepted the positions come from pq (the same x, y, z; its w, (2h)^2, is then unused), which the density
// scan has just read for the same candidates, so the loads tend to hit L1.
template <bool kPeriodic, bool kAccepted = false>
__device__ __forceinline__ void density_pair(const StepArgs& a, float4 pi, uint32_t j1, float s1x, float s1y,
                                             float s1z, uint32_t j2, float s2x, float s2y, float s2z, float& rho) {
    const float4* pos = kAccepted ? a.pq : a.ph;
    const float4 p1 = __ldg(pos + j1), p2 = __ldg(pos + j2);
    const float4 k1 = __ldg(a.kc + j1), k2 = __ldg(a.kc + j2);
    float2 x = make_float2(p1.x, p2.x), y = make_float2(p1.y, p2.y), z = make_float2(p1.z, p2.z);
    if (kPeriodic) {
        x = __fadd2_rn(x, make_float2(s1x, s2x));
        y = __fadd2_rn(y, make_float2(s1y, s2y));
        z = __fadd2_rn(z, make_float2(s1z, s2z));
    }
    const float2 dx = __fadd2_rn(x, make_float2(-pi.x, -pi.x));
    const float2 dy = __fadd2_rn(y, make_float2(-pi.y, -pi.y));
    const float2 dz = __fadd2_rn(z, make_float2(-pi.z, -pi.z));
    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    const float2 h = make_float2(p1.w, p2.w);
    const float2 twoh = __fadd2_rn(h, h);
    const float2 t2h = __fmul2_rn(twoh, twoh);
    const float2 r = make_float2(sqrtf(r2.x), sqrtf(r2.y));
    // kernel_w(r, 1/h, coef/h^3) for both
    const float2 q = __fmul2_rn(r, make_float2(k1.x, k2.x));
    const float2 t = __ffma2_rn(make_float2(-0.5f, -0.5f), q, make_float2(1.0f, 1.0f));
    const float2 tt = __fmul2_rn(t, t);
    const float2 t4 = __fmul2_rn(tt, tt);
    const float2 w = __fmul2_rn(__fmul2_rn(make_float2(k1.y, k2.y), t4),
                                __ffma2_rn(make_float2(2.0f, 2.0f), q, make_float2(1.0f, 1.0f)));
    if (kAccepted || r2.x <= t2h.x) rho = fmaf(k1.w, q.x > 2.0f ? 0.0f : w.x, rho);
    if (kAccepted || r2.y <= t2h.y) rho = fmaf(k2.w, q.y > 2.0f ? 0.0f : w.y, rho);
}

// Boundary density of particle i over the cells of lane `lane` (BoundaryAlgorithm.cu:15-51).
template <int kLanes>
__device__ __forceinline__ float boundary_density(const StepArgs& a, const BoundaryDev& b, uint32_t i, float4 pi,
                                                  int lane) {
    const float R = pi.w + pi.w;
    const float4 ki = a.kc[i];
    const float cut = R * R;
    const bool periodic = a.grid.periodic;
    float rb = 0.0f;
    for_each_boundary_cell<kLanes>(
        a.grid, b, pi.x, pi.y, pi.z, R, lane,
        [&](uint32_t kb, uint32_t ke, float shx, float shy, float shz) {
            for (uint32_t k = kb + lane; k < ke; k += kLanes) {
                const float4 pb = __ldg(b.pos + k);
                const float xb = periodic ? pb.x + shx : pb.x;
                const float yb = periodic ? pb.y + shy : pb.y;
                const float zb = periodic ? pb.z + shz : pb.z;
                const float dx = xb - pi.x, dy = yb - pi.y, dz = zb - pi.z;
                const float r2 = dist2(dx, dy, dz);
                if (r2 > cut) continue;
                const float w = kernel_w(sqrtf(r2), ki.x, ki.y);
                rb = fmaf(pb.w, w, rb);
            }
        });
    return rb;
}

// Accumulators of the force pass: pressure, viscosity, cohesion; boundary pressure, boundary friction.
struct ForceAcc {
    float ap[3], av[3], as[3], bp[3], bf[3];
};

// boundary_density<1> that also records, after the fluid entries of the particle's row, one entry per block of up
// to 32 wall members with an accepted member: (first member | image code << 27, acceptance mask). `space` entries
// fit; *entries is their number, or kBoundaryWalk when they did not fit (the force pass then walks the cells).
__device__ __forceinline__ float boundary_density_rows(const StepArgs& a, const BoundaryDev& b, uint32_t i, float4 pi,
                                                       uint2* out, uint32_t space, uint32_t* entries) {
    const float R = pi.w + pi.w;
    const float4 ki = a.kc[i];
    const float cut = R * R;
    const bool periodic = a.grid.periodic;
    float rb = 0.0f;
    uint32_t n = 0;
    for_each_boundary_cell<1>(
        a.grid, b, pi.x, pi.y, pi.z, R, 0, [&](uint32_t kb, uint32_t ke, float shx, float shy, float shz) {
            const uint32_t code = periodic ? (shift_code(shx, shy, shz) << kIdxBits) : 0u;
            for (uint32_t c0 = kb; c0 < ke; c0 += 32u) {
                const uint32_t cn = ke - c0 < 32u ? ke - c0 : 32u;
                uint32_t mask = 0;
                for (uint32_t k = 0; k < cn; ++k) {
                    const float4 pb = __ldg(b.pos + c0 + k);
                    const float xb = periodic ? pb.x + shx : pb.x;
                    const float yb = periodic ? pb.y + shy : pb.y;
                    const float zb = periodic ? pb.z + shz : pb.z;
                    const float dx = xb - pi.x, dy = yb - pi.y, dz = zb - pi.z;
                    const float r2 = dist2(dx, dy, dz);
                    if (r2 > cut) continue;
                    const float w = kernel_w(sqrtf(r2), ki.x, ki.y);
                    rb = fmaf(pb.w, w, rb);
                    mask |= 1u << k;
                }
                if (mask != 0u) {
                    if (n < space) out[n] = make_uint2(c0 | code, mask);
                    n++;
                }
            }
        });
    *entries = n <= space ? n : kBoundaryWalk;
    return rb;
}

struct ForceCtx {
    float4 pi, vi;
    float rhoi, pti, Ki, ei, hi;
    bool visc_on, sigma_on;
};

__device__ __forceinline__ ForceCtx force_ctx(const StepArgs& a, uint32_t i) {
    ForceCtx c;
    c.pi = a.ph[i];
    c.vi = a.vm[i];
    const float2 rpi = a.rp[i];
    c.hi = c.pi.w;
    c.rhoi = rpi.x;
    c.pti = rpi.y;
    c.Ki = ((2.0f * a.phys.alpha) * c.hi) * a.phys.c0;
    c.ei = (0.01f * c.hi) * c.hi;
    c.visc_on = a.phys.visc_on;
    c.sigma_on = a.phys.sigma_on;
    return c;
}

// Pressure, viscosity and cohesion terms of fluid neighbour j (Algorithm.cu:56-221).
template <bool kMorris, bool kSigma = true>
__device__ __forceinline__ void force_term(const StepArgs& a, const ForceCtx& c, uint32_t j, float shx, float shy,
                                           float shz, ForceAcc& f) {
    const bool periodic = a.grid.periodic;
    const float4 pj = __ldg(a.ph + j);
    const float xj = periodic ? pj.x + shx : pj.x;
    const float yj = periodic ? pj.y + shy : pj.y;
    const float zj = periodic ? pj.z + shz : pj.z;
    const float dx = c.pi.x - xj, dy = c.pi.y - yj, dz = c.pi.z - zj;
    const float r2 = dist2(dx, dy, dz);
    const float twoh = pj.w + pj.w;
    if (r2 > twoh * twoh) return;
    const float4 fj = __ldg(a.fr + j);  // rho, p/rho^2, 1/h, dcoef/h^4
    const float4 vj = __ldg(a.vm + j);  // v, m
    const float r = sqrtf(r2);
    float u[3];
    if (r > 0.0f) {
        const float ir = 1.0f / r;
        u[0] = dx * ir;
        u[1] = dy * ir;
        u[2] = dz * ir;
    } else {
        u[0] = 0.0f;
        u[1] = 1.0f;
        u[2] = 0.0f;
    }
    const float dw = kernel_dw(r, fj.z, fj.w);
    const float mj = vj.w;
    {
        const float sp = (mj * dw) * (c.pti + fj.y);
#pragma unroll
        for (int q = 0; q < 3; q++) f.ap[q] = fmaf(-sp, u[q], f.ap[q]);
    }
    if (c.visc_on) {
        const float vd[3] = {c.vi.x - vj.x, c.vi.y - vj.y, c.vi.z - vj.z};
        const float rhoj = fj.x;
        if (!kMorris) {
            const float comp = fmaf(vd[2], dz, fmaf(vd[1], dy, vd[0] * dx));
            if (comp < 0.0f) {
                const float nuij = c.Ki / (c.rhoi + rhoj);
                const float piv = (-nuij * comp) / (r2 + c.ei);
                const float sv = (mj * piv) * dw;
#pragma unroll
                for (int q = 0; q < 3; q++) f.av[q] = fmaf(-sv, u[q], f.av[q]);
            }
        } else {
            const float coef = ((mj * a.phys.nu) * (c.rhoi + rhoj)) / (c.rhoi * rhoj);
            const float sv = coef * ((r * dw) / (r2 + c.ei));
#pragma unroll
            for (int q = 0; q < 3; q++) f.av[q] = fmaf(sv, vd[q], f.av[q]);
        }
    }
    if (kSigma && c.sigma_on) {
        const float4 kj = __ldg(a.kc + j);
        const float ss = mj * kernel_w(r, kj.x, kj.y);
#pragma unroll
        for (int q = 0; q < 3; q++) f.as[q] = fmaf(ss, u[q], f.as[q]);
    }
}

// force_term for two neighbours: the per-pair quantities in packed FP32x2 arithmetic (each half rounds as the
// scalar operation; divisions and square roots stay scalar), each accumulator updated for j1, then j2.
template <bool kMorris, bool kPeriodic, bool kSigma = true, bool kAccepted = false>
__device__ __forceinline__ void force_pair(const StepArgs& a, const ForceCtx& c, uint32_t j1, float s1x, float s1y,
                                           float s1z, uint32_t j2, float s2x, float s2y, float s2z, ForceAcc& f) {
    const float4 p1 = __ldg(a.ph + j1), p2 = __ldg(a.ph + j2);
    const float4 f1 = __ldg(a.fr + j1), f2 = __ldg(a.fr + j2);  // rho, p/rho^2, 1/h, dcoef/h^4
    const float4 v1 = __ldg(a.vm + j1), v2 = __ldg(a.vm + j2);  // v, m
    float2 x = make_float2(p1.x, p2.x), y = make_float2(p1.y, p2.y), z = make_float2(p1.z, p2.z);
    if (kPeriodic) {
        x = __fadd2_rn(x, make_float2(s1x, s2x));
        y = __fadd2_rn(y, make_float2(s1y, s2y));
        z = __fadd2_rn(z, make_float2(s1z, s2z));
    }
    // d = p_i - p_j
    const float2 dx = __fadd2_rn(make_float2(c.pi.x, c.pi.x), make_float2(-x.x, -x.y));
    const float2 dy = __fadd2_rn(make_float2(c.pi.y, c.pi.y), make_float2(-y.x, -y.y));
    const float2 dz = __fadd2_rn(make_float2(c.pi.z, c.pi.z), make_float2(-z.x, -z.y));
    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    const float2 h = make_float2(p1.w, p2.w);
    const float2 twoh = __fadd2_rn(h, h);
    const float2 t2h = __fmul2_rn(twoh, twoh);
    const bool ok1 = kAccepted || r2.x <= t2h.x, ok2 = kAccepted || r2.y <= t2h.y;
    const float2 r = make_float2(sqrtf(r2.x), sqrtf(r2.y));
    const float2 ir = make_float2(r.x > 0.0f ? 1.0f / r.x : 0.0f, r.y > 0.0f ? 1.0f / r.y : 0.0f);
    float2 ux = __fmul2_rn(dx, ir), uy = __fmul2_rn(dy, ir), uz = __fmul2_rn(dz, ir);
    if (!(r.x > 0.0f)) {
        ux.x = 0.0f;
        uy.x = 1.0f;
        uz.x = 0.0f;
    }
    if (!(r.y > 0.0f)) {
        ux.y = 0.0f;
        uy.y = 1.0f;
        uz.y = 0.0f;
    }
    // kernel_dw(r, 1/h, dcoef/h^4)
    const float2 q = __fmul2_rn(r, make_float2(f1.z, f2.z));
    const float2 t = __ffma2_rn(make_float2(-0.5f, -0.5f), q, make_float2(1.0f, 1.0f));
    const float2 t3 = __fmul2_rn(__fmul2_rn(t, t), t);
    float2 dw = __fmul2_rn(__fmul2_rn(make_float2(f1.w, f2.w), q), t3);
    if (q.x > 2.0f) dw.x = 0.0f;
    if (q.y > 2.0f) dw.y = 0.0f;
    const float2 m = make_float2(v1.w, v2.w);
    const float2 sp = __fmul2_rn(__fmul2_rn(m, dw), __fadd2_rn(make_float2(c.pti, c.pti), make_float2(f1.y, f2.y)));
    if (ok1) {
        f.ap[0] = fmaf(-sp.x, ux.x, f.ap[0]);
        f.ap[1] = fmaf(-sp.x, uy.x, f.ap[1]);
        f.ap[2] = fmaf(-sp.x, uz.x, f.ap[2]);
    }
    if (ok2) {
        f.ap[0] = fmaf(-sp.y, ux.y, f.ap[0]);
        f.ap[1] = fmaf(-sp.y, uy.y, f.ap[1]);
        f.ap[2] = fmaf(-sp.y, uz.y, f.ap[2]);
    }
    if (c.visc_on) {
        const float2 vdx = __fadd2_rn(make_float2(c.vi.x, c.vi.x), make_float2(-v1.x, -v2.x));
        const float2 vdy = __fadd2_rn(make_float2(c.vi.y, c.vi.y), make_float2(-v1.y, -v2.y));
        const float2 vdz = __fadd2_rn(make_float2(c.vi.z, c.vi.z), make_float2(-v1.z, -v2.z));
        const float2 rhoj = make_float2(f1.x, f2.x);
        const float2 den = __fadd2_rn(r2, make_float2(c.ei, c.ei));
        if (!kMorris) {
            const float2 comp = __ffma2_rn(vdz, dz, __ffma2_rn(vdy, dy, __fmul2_rn(vdx, dx)));
            const float2 rsum = __fadd2_rn(make_float2(c.rhoi, c.rhoi), rhoj);
            if (ok1 && comp.x < 0.0f) {
                const float nuij = c.Ki / rsum.x;
                const float piv = (-nuij * comp.x) / den.x;
                const float sv = (m.x * piv) * dw.x;
                f.av[0] = fmaf(-sv, ux.x, f.av[0]);
                f.av[1] = fmaf(-sv, uy.x, f.av[1]);
                f.av[2] = fmaf(-sv, uz.x, f.av[2]);
            }
            if (ok2 && comp.y < 0.0f) {
                const float nuij = c.Ki / rsum.y;
                const float piv = (-nuij * comp.y) / den.y;
                const float sv = (m.y * piv) * dw.y;
                f.av[0] = fmaf(-sv, ux.y, f.av[0]);
                f.av[1] = fmaf(-sv, uy.y, f.av[1]);
                f.av[2] = fmaf(-sv, uz.y, f.av[2]);
            }
        } else {
            const float2 mnu = __fmul2_rn(m, make_float2(a.phys.nu, a.phys.nu));
            const float2 num = __fmul2_rn(mnu, __fadd2_rn(make_float2(c.rhoi, c.rhoi), rhoj));
            const float2 prod = __fmul2_rn(make_float2(c.rhoi, c.rhoi), rhoj);
            const float2 rdw = __fmul2_rn(r, dw);
            if (ok1) {
                const float sv = (num.x / prod.x) * (rdw.x / den.x);
                f.av[0] = fmaf(sv, vdx.x, f.av[0]);
                f.av[1] = fmaf(sv, vdy.x, f.av[1]);
                f.av[2] = fmaf(sv, vdz.x, f.av[2]);
            }
            if (ok2) {
                const float sv = (num.y / prod.y) * (rdw.y / den.y);
                f.av[0] = fmaf(sv, vdx.y, f.av[0]);
                f.av[1] = fmaf(sv, vdy.y, f.av[1]);
                f.av[2] = fmaf(sv, vdz.y, f.av[2]);
            }
        }
    }
    if (kSigma && c.sigma_on) {
        const float4 k1 = __ldg(a.kc + j1), k2 = __ldg(a.kc + j2);
        if (ok1) {
            const float ss = m.x * kernel_w(r.x, k1.x, k1.y);
            f.as[0] = fmaf(ss, ux.x, f.as[0]);
            f.as[1] = fmaf(ss, uy.x, f.as[1]);
            f.as[2] = fmaf(ss, uz.x, f.as[2]);
        }
        if (ok2) {
            const float ss = m.y * kernel_w(r.y, k2.x, k2.y);
            f.as[0] = fmaf(ss, ux.y, f.as[0]);
            f.as[1] = fmaf(ss, uy.y, f.as[1]);
            f.as[2] = fmaf(ss, uz.y, f.as[2]);
        }
    }
}

// Boundary pressure and friction (BoundaryAlgorithm.cu:53-162) over the cells of lane `lane`.
template <int kLanes>
__device__ __forceinline__ void boundary_forces(const StepArgs& a, const BoundaryDev& b, uint32_t i,
                                                const ForceCtx& c, ForceAcc& f, int lane) {
    const float R = c.hi + c.hi;
    const float4 ki = a.kc[i];
    const float cut = R * R;
    const bool periodic = a.grid.periodic;
    const float c0 = a.phys.c0;
    for_each_boundary_cell<kLanes>(
        a.grid, b, c.pi.x, c.pi.y, c.pi.z, R, lane,
        [&](uint32_t kb, uint32_t ke, float shx, float shy, float shz) {
            for (uint32_t k = kb + lane; k < ke; k += kLanes) {
                const float4 pb = __ldg(b.pos + k);
                const float xb = periodic ? pb.x + shx : pb.x;
                const float yb = periodic ? pb.y + shy : pb.y;
                const float zb = periodic ? pb.z + shz : pb.z;
                const float dx = c.pi.x - xb, dy = c.pi.y - yb, dz = c.pi.z - zb;
                const float r2 = dist2(dx, dy, dz);
                if (r2 > cut) continue;
                const float r = sqrtf(r2);
                float u[3];
                if (r > 0.0f) {
                    const float ir = 1.0f / r;
                    u[0] = dx * ir;
                    u[1] = dy * ir;
                    u[2] = dz * ir;
                } else {
                    u[0] = 0.0f;
                    u[1] = 1.0f;
                    u[2] = 0.0f;
                }
                const float dw = kernel_dw(r, ki.x, ki.z);
                const float psi = pb.w;
                const float sp = (psi * c.pti) * dw;
#pragma unroll
                for (int q = 0; q < 3; q++) f.bp[q] = fmaf(-sp, u[q], f.bp[q]);
                const float comp = fmaf(c.vi.z, dz, fmaf(c.vi.y, dy, c.vi.x * dx));
                if (comp < 0.0f) {
                    const float nub = ((__ldg(b.fric + k) * c.hi) * c0) / (2.0f * c.rhoi);
                    const float pib = (-nub * comp) / (r2 + c.ei);
                    const float sf = (psi * pib) * dw;
#pragma unroll
                    for (int q = 0; q < 3; q++) f.bf[q] = fmaf(-sf, u[q], f.bf[q]);
                }
            }
        });
}

// a = g + pressure + viscosity + cohesion + boundary pressure + boundary friction, in the reference's kernel order.
__device__ __forceinline__ void finish_force(const StepArgs& a, uint32_t i, const ForceCtx& c, const ForceAcc& f) {
    float acc[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
        float v = a.phys.gravity[q];
        v = v + f.ap[q];
        if (c.visc_on) v = v + f.av[q];
        if (c.sigma_on) v = v + (a.phys.sigma / c.vi.w) * f.as[q];
        v = v + f.bp[q];
        v = v + f.bf[q];
        acc[q] = v;
    }
    if (!(isfinite(acc[0]) && isfinite(acc[1]) && isfinite(acc[2]))) atomicOr(a.err, 0x2u);
    a.acc[i] = make_float4(acc[0], acc[1], acc[2], 0.0f);
}

template <bool kCull, class Body>
__device__ __forceinline__ void fluid_candidates(const StepArgs& a, const CellsDev& c, float4 pi, Body&& body) {
    const float R = pi.w + pi.w;
    for_each_cell<kCull>(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], pi.x, pi.y, pi.z, R, 0.0f,
                         body);
}

}  // namespace

// Boundary pressure and friction term of wall member k (Algorithm.cu:118-221), the member known to be within the
// support: the arithmetic of boundary_forces.
__device__ __forceinline__ void boundary_term(const StepArgs& a, const BoundaryDev& b, const ForceCtx& c, float4 ki,
                                              uint32_t k, float shx, float shy, float shz, ForceAcc& f) {
    const bool periodic = a.grid.periodic;
    const float4 pb = __ldg(b.pos + k);
    const float xb = periodic ? pb.x + shx : pb.x;
    const float yb = periodic ? pb.y + shy : pb.y;
    const float zb = periodic ? pb.z + shz : pb.z;
    const float dx = c.pi.x - xb, dy = c.pi.y - yb, dz = c.pi.z - zb;
    const float r2 = dist2(dx, dy, dz);
    const float r = sqrtf(r2);
    float u[3];
    if (r > 0.0f) {
        const float ir = 1.0f / r;
        u[0] = dx * ir;
        u[1] = dy * ir;
        u[2] = dz * ir;
    } else {
        u[0] = 0.0f;
        u[1] = 1.0f;
        u[2] = 0.0f;
    }
    const float dw = kernel_dw(r, ki.x, ki.z);
    const float psi = pb.w;
    const float sp = (psi * c.pti) * dw;
#pragma unroll
    for (int q = 0; q < 3; q++) f.bp[q] = fmaf(-sp, u[q], f.bp[q]);
    const float comp = fmaf(c.vi.z, dz, fmaf(c.vi.y, dy, c.vi.x * dx));
    if (comp < 0.0f) {
        const float nub = ((__ldg(b.fric + k) * c.hi) * a.phys.c0) / (2.0f * c.rhoi);
        const float pib = (-nub * comp) / (r2 + c.ei);
        const float sf = (psi * pib) * dw;
#pragma unroll
        for (int q = 0; q < 3; q++) f.bf[q] = fmaf(-sf, u[q], f.bf[q]);
    }
}

// boundary_term for two wall members in packed FP32x2 arithmetic (each half rounds as the scalar operation; divisions
// and square roots stay scalar); each accumulator is updated for k1, then k2.
__device__ __forceinline__ void boundary_pair(const StepArgs& a, const BoundaryDev& b, const ForceCtx& c, float4 ki,
                                              uint32_t k1, float s1x, float s1y, float s1z, uint32_t k2, float s2x,
                                              float s2y, float s2z, ForceAcc& f) {
    const float4 p1 = __ldg(b.pos + k1), p2 = __ldg(b.pos + k2);
    float2 x = make_float2(p1.x, p2.x), y = make_float2(p1.y, p2.y), z = make_float2(p1.z, p2.z);
    if (a.grid.periodic) {
        x = __fadd2_rn(x, make_float2(s1x, s2x));
        y = __fadd2_rn(y, make_float2(s1y, s2y));
        z = __fadd2_rn(z, make_float2(s1z, s2z));
    }
    const float2 dx = __fadd2_rn(make_float2(c.pi.x, c.pi.x), make_float2(-x.x, -x.y));
    const float2 dy = __fadd2_rn(make_float2(c.pi.y, c.pi.y), make_float2(-y.x, -y.y));
    const float2 dz = __fadd2_rn(make_float2(c.pi.z, c.pi.z), make_float2(-z.x, -z.y));
    const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    const float2 r = make_float2(sqrtf(r2.x), sqrtf(r2.y));
    const float2 ir = make_float2(r.x > 0.0f ? 1.0f / r.x : 0.0f, r.y > 0.0f ? 1.0f / r.y : 0.0f);
    float2 ux = __fmul2_rn(dx, ir), uy = __fmul2_rn(dy, ir), uz = __fmul2_rn(dz, ir);
    if (!(r.x > 0.0f)) {
        ux.x = 0.0f;
        uy.x = 1.0f;
        uz.x = 0.0f;
    }
    if (!(r.y > 0.0f)) {
        ux.y = 0.0f;
        uy.y = 1.0f;
        uz.y = 0.0f;
    }
    // kernel_dw(r, 1/h_i, dcoef/h_i^4)
    const float2 q = __fmul2_rn(r, make_float2(ki.x, ki.x));
    const float2 t = __ffma2_rn(make_float2(-0.5f, -0.5f), q, make_float2(1.0f, 1.0f));
    const float2 t3 = __fmul2_rn(__fmul2_rn(t, t), t);
    float2 dw = __fmul2_rn(__fmul2_rn(make_float2(ki.z, ki.z), q), t3);
    if (q.x > 2.0f) dw.x = 0.0f;
    if (q.y > 2.0f) dw.y = 0.0f;
    const float2 psi = make_float2(p1.w, p2.w);
    const float2 sp = __fmul2_rn(__fmul2_rn(psi, make_float2(c.pti, c.pti)), dw);
    f.bp[0] = fmaf(-sp.x, ux.x, f.bp[0]);
    f.bp[1] = fmaf(-sp.x, uy.x, f.bp[1]);
    f.bp[2] = fmaf(-sp.x, uz.x, f.bp[2]);
    f.bp[0] = fmaf(-sp.y, ux.y, f.bp[0]);
    f.bp[1] = fmaf(-sp.y, uy.y, f.bp[1]);
    f.bp[2] = fmaf(-sp.y, uz.y, f.bp[2]);
    const float2 comp = __ffma2_rn(make_float2(c.vi.z, c.vi.z), dz,
                                   __ffma2_rn(make_float2(c.vi.y, c.vi.y), dy, __fmul2_rn(make_float2(c.vi.x, c.vi.x), dx)));
    if (comp.x < 0.0f) {
        const float nub = ((__ldg(b.fric + k1) * c.hi) * a.phys.c0) / (2.0f * c.rhoi);
        const float pib = (-nub * comp.x) / (r2.x + c.ei);
        const float sf = (psi.x * pib) * dw.x;
        f.bf[0] = fmaf(-sf, ux.x, f.bf[0]);
        f.bf[1] = fmaf(-sf, uy.x, f.bf[1]);
        f.bf[2] = fmaf(-sf, uz.x, f.bf[2]);
    }
    if (comp.y < 0.0f) {
        const float nub = ((__ldg(b.fric + k2) * c.hi) * a.phys.c0) / (2.0f * c.rhoi);
        const float pib = (-nub * comp.y) / (r2.y + c.ei);
        const float sf = (psi.y * pib) * dw.y;
        f.bf[0] = fmaf(-sf, ux.y, f.bf[0]);
        f.bf[1] = fmaf(-sf, uy.y, f.bf[1]);
        f.bf[2] = fmaf(-sf, uz.y, f.bf[2]);
    }
}

// Boundary forces of particle i from its recorded wall entries, in the recorded (canonical) order.
__device__ __forceinline__ void boundary_forces_rows(const StepArgs& a, const BoundaryDev& b, uint32_t i,
                                                     const ForceCtx& c, ForceAcc& f, const uint2* ent, uint32_t n) {
    const float4 ki = a.kc[i];
    uint32_t e = 0, first = 0, mask = 0;
    float shx = 0.0f, shy = 0.0f, shz = 0.0f;
    auto pull = [&](uint32_t& k, float& sx, float& sy, float& sz) -> bool {
        if (mask == 0u) {
            if (e >= n) return false;
            row_entry(a.grid, __ldg(ent + e), first, mask, shx, shy, shz);
            e++;
        }
        k = first + (uint32_t)(__ffs(mask) - 1);
        mask &= mask - 1u;
        sx = shx;
        sy = shy;
        sz = shz;
        return true;
    };
    for (;;) {
        uint32_t k1, k2;
        float s1x, s1y, s1z, s2x, s2y, s2z;
        if (!pull(k1, s1x, s1y, s1z)) break;
        if (!pull(k2, s2x, s2y, s2z)) {
            boundary_term(a, b, c, ki, k1, s1x, s1y, s1z, f);
            break;
        }
        boundary_pair(a, b, c, ki, k1, s1x, s1y, s1z, k2, s2x, s2y, s2z, f);
    }
}

// Density pass, ordinary particles; heavy particles are queued for k_density_heavy.
// The bodies of the neighbour kernels are device functions so that the per-simulation kernels and the segmented
// (multi-scene) kernels run the same code: particle i (ordinary), or the queued particle of warp item w (heavy,
// long row). The warp-level parts need all 32 lanes of a warp to enter together.
template <bool kPeriodic>
__device__ __forceinline__ void density_ordinary(const StepArgs& a, const CellsDev& c, const BoundaryDev& b,
                                                 const NbrDev& nl, const uint32_t i) {
    bool in = i < count_of(a);
    if (in && i >= nl.rows) {
        atomicOr(a.err, 0x10u);  // rows not grown for this count: the particle is skipped, the step flagged
        in = false;
    }
    const float4 pi = in ? a.ph[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float R = pi.w + pi.w;
    bool active = in;
    if (in && box_cells(a.grid, pi, R) > kHeavyCells) active = false;  // k_density_heavy (sets cnt[i])
    constexpr bool periodic = kPeriodic;
    uint2* row = nl.ent + (size_t)(in ? i : 0) * nl.maxe;
    const uint32_t maxe = nl.maxe;
    uint32_t cnt = 0;
    // entries are written in 16-byte pairs: an even entry waits in registers for its odd partner
    uint2 held = make_uint2(0u, 0u);
    float rho = 0.0f;
    auto append = [&](uint32_t first, uint32_t mask) {
        if (cnt < maxe) {
            if (cnt & 1u)
                *reinterpret_cast<uint4*>(row + (cnt - 1u)) = make_uint4(held.x, held.y, first, mask);
            else
                held = make_uint2(first, mask);
        }
        cnt++;
    };
    // Per block of up to 32 members of a sub-cell: a support test of every member builds the lane's acceptance
    // mask, and the block (first member, mask) goes to the lane's list row. The kernel sums are formed afterwards
    // from the row, one accepted neighbour per iteration.
    const float2 nx = make_float2(-pi.x, -pi.x), ny = make_float2(-pi.y, -pi.y), nz = make_float2(-pi.z, -pi.z);
    auto scan_block = [&](uint32_t c0, uint32_t cn, uint32_t code, float shx, float shy, float shz) {
        // members from last to first, so the mask is built by shifts: bit k = member c0 + k. Two members per
        // iteration in packed FP32x2 arithmetic (each half rounds exactly as the scalar operation would).
        uint32_t mask = 0;
        int k = (int)cn - 1;
        if ((cn & 1u) != 0u) {
            const float4 pj = __ldg(a.pq + c0 + k);
            const float xj = periodic ? pj.x + shx : pj.x;
            const float yj = periodic ? pj.y + shy : pj.y;
            const float zj = periodic ? pj.z + shz : pj.z;
            const float dx = xj - pi.x, dy = yj - pi.y, dz = zj - pi.z;
            const float r2 = dist2(dx, dy, dz);
            mask = r2 <= pj.w ? 1u : 0u;
            --k;
        }
#pragma unroll 2
        for (; k >= 1; k -= 2) {
            const float4 p1 = __ldg(a.pq + c0 + k), p0 = __ldg(a.pq + c0 + k - 1);
            float2 x = make_float2(p1.x, p0.x), y = make_float2(p1.y, p0.y), z = make_float2(p1.z, p0.z);
            if (periodic) {
                x = __fadd2_rn(x, make_float2(shx, shx));
                y = __fadd2_rn(y, make_float2(shy, shy));
                z = __fadd2_rn(z, make_float2(shz, shz));
            }
            const float2 dx = __fadd2_rn(x, nx), dy = __fadd2_rn(y, ny), dz = __fadd2_rn(z, nz);
            const float2 r2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
            mask = (mask << 2) | (r2.x <= p1.w ? 2u : 0u) | (r2.y <= p0.w ? 1u : 0u);
        }
        if (mask != 0u) append(c0 | code, mask);
    };
    auto scan = [&](uint32_t jb, uint32_t je, float shx, float shy, float shz, bool need) {
        if (!need) return;
        const uint32_t code = periodic ? (shift_code(shx, shy, shz) << kIdxBits) : 0u;
        for (uint32_t c0 = jb; c0 < je; c0 += 32) scan_block(c0, je - c0 < 32u ? je - c0 : 32u, code, shx, shy, shz);
    };
    // the warp's 32 particles are neighbours in the cell order: walk the union of their boxes together
    const bool together = for_each_cell_warp(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], active,
                                             pi.x, pi.y, pi.z, R, kMaxUnion, scan);
    if (!together && active)
        fluid_candidates<true>(a, c, pi, [&](uint32_t jb, uint32_t je, float shx, float shy, float shz) {
            scan(jb, je, shx, shy, shz, true);
        });
    if (!active) return;
    nl.cnt[i] = cnt;
    if (cnt > maxe) {  // row overflowed: density and forces by the warp kernels
        nl.dover[atomicAdd(nl.dover_n, 1u)] = i;
        return;
    }
    if (cnt & 1u) row[cnt - 1u] = held;  // the unpaired last entry
    if (cnt > kRowHeavy) {  // many neighbours: summed over the row by a warp (k_density_row)
        nl.drow[atomicAdd(nl.drow_n, 1u)] = i;
        return;
    }
    // the fluid sum over the row in canonical order (plain loads: the row was written by this thread), two
    // neighbours per iteration in packed FP32x2 arithmetic, added to rho one after the other
    {
        uint2 next = cnt > 0u ? row[0] : make_uint2(0u, 0u);
        uint32_t k = 1, first = 0, mask = 0;
        float shx = 0.0f, shy = 0.0f, shz = 0.0f;
        auto pull = [&](uint32_t& j, float& sx, float& sy, float& sz) -> bool {
            if (mask == 0u) {
                if (k > cnt) return false;
                decode_entry(a.grid, next.x, first, shx, shy, shz);
                mask = next.y;
                if (k < cnt) next = row[k];
                k++;
            }
            j = first + (uint32_t)(__ffs(mask) - 1);
            mask &= mask - 1u;
            sx = shx;
            sy = shy;
            sz = shz;
            return true;
        };
        for (;;) {
            uint32_t j1, j2;
            float s1x, s1y, s1z, s2x, s2y, s2z;
            if (!pull(j1, s1x, s1y, s1z)) break;
            if (!pull(j2, s2x, s2y, s2z)) {
                density_term_accepted(a, pi, j1, s1x, s1y, s1z, rho);
                break;
            }
            density_pair<periodic, true>(a, pi, j1, s1x, s1y, s1z, j2, s2x, s2y, s2z, rho);
        }
    }
    float rb = 0.0f;
    uint32_t bn = 0;
    if (b.n != 0) rb = boundary_density_rows(a, b, i, pi, row + cnt, maxe - cnt, &bn);
    nl.bcnt[i] = bn;
    const float rh = rho + rb;
    if (!isfinite(rh)) atomicOr(a.err, 0x2u);
    const float pt = pressure_term(rh, a.phys.rho0, a.phys.B);
    a.rp[i] = make_float2(rh, pt);
    const float4 ki = a.kc[i];
    a.fr[i] = make_float4(rh, pt, ki.x, ki.z);
}

template <bool kPeriodic>
__global__ void __launch_bounds__(128, 7) k_density(StepArgs a, CellsDev c, BoundaryDev b, NbrDev nl) {
    density_ordinary<kPeriodic>(a, c, b, nl, blockIdx.x * blockDim.x + threadIdx.x);
}

// Density of one heavy particle (queue position w, particle i) by one warp.
__device__ __forceinline__ void density_heavy_item(const StepArgs& a, const CellsDev& c, const BoundaryDev& b,
                                                   const NbrDev& nl, const uint32_t w, const uint32_t i,
                                                   const bool pooled, const int lane) {
    const bool periodic = a.grid.periodic;
    {
        const float4 pi = a.ph[i];
        const float R = pi.w + pi.w;
        const bool keep = pooled && w < nl.pool_slots;
        uint2* seg = keep ? nl.pool + ((size_t)w * 32 + lane) * kPoolLaneEntries : nullptr;
        uint32_t kept = 0;
        float rho = 0.0f;
        for_each_subcell_lane(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], pi.x, pi.y, pi.z, R, 0.0f, lane,
                              [&](uint32_t jb, uint32_t je, float shx, float shy, float shz) {
                                  const uint32_t code = periodic ? (shift_code(shx, shy, shz) << kIdxBits) : 0u;
                                  for (uint32_t c0 = jb; c0 < je; c0 += 32) {
                                      const uint32_t cn = je - c0 < 32u ? je - c0 : 32u;
                                      uint32_t mask = 0;
                                      for (int k = (int)cn - 1; k >= 0; --k)
                                          mask = (mask << 1) |
                                                 (supported(a.grid, pi, __ldg(a.ph + c0 + k), shx, shy, shz) ? 1u : 0u);
                                      if (mask == 0u) continue;
                                      if (keep) {
                                          if (kept < kPoolLaneEntries) seg[kept] = make_uint2(c0 | code, mask);
                                          kept++;
                                      }
                                      while (mask != 0u) {
                                          const uint32_t k = (uint32_t)(__ffs(mask) - 1);
                                          mask &= mask - 1u;
                                          density_term(a, pi, c0 + k, shx, shy, shz, rho);
                                      }
                                  }
                              });
        if (pooled) {
            const bool fits = keep && !__any_sync(0xffffffffu, kept > kPoolLaneEntries);
            if (fits) nl.pool_cnt[(size_t)w * 32 + lane] = kept;
            if (lane == 0) nl.cnt[i] = fits ? (kPooled | w) : kHeavyMark;
        }
        rho = warp_sum_butterfly(rho);
        float rb = 0.0f;
        if (b.n != 0) rb = warp_sum_butterfly(boundary_density<32>(a, b, i, pi, lane));
        if (lane == 0) {
            const float rh = rho + rb;
            if (!isfinite(rh)) atomicOr(a.err, 0x2u);
            const float pt = pressure_term(rh, a.phys.rho0, a.phys.B);
            a.rp[i] = make_float2(rh, pt);
            const float4 ki = a.kc[i];
            a.fr[i] = make_float4(rh, pt, ki.x, ki.z);
            nl.fheavy[atomicAdd(nl.fheavy_n, 1u)] = i;
        }
    }
}

// Density of the heavy particles: one warp per particle.
__global__ void __launch_bounds__(128, 2) k_density_heavy(StepArgs a, CellsDev c, BoundaryDev b, NbrDev nl,
                                                          const uint32_t* queue, const uint32_t* queue_n, bool pooled) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nh = *queue_n;
    for (uint32_t w = warp; w < nh; w += nwarps) density_heavy_item(a, c, b, nl, w, queue[w], pooled, lane);
}

// Force pass, ordinary particles: walks the particle's neighbour list. Heavy particles and particles whose row
// overflowed are left to k_forces_heavy.
template <bool kMorris, bool kSigma>
__device__ __forceinline__ void forces_ordinary(const StepArgs& a, const CellsDev& c, const BoundaryDev& b,
                                                const NbrDev& nl, const uint32_t i) {
    if (i >= count_of(a) || i >= nl.rows) return;
    const uint32_t cnt = nl.cnt[i];
    if (cnt > kRowHeavy) return;  // long row (k_forces_row), overflowed or heavy (k_forces_heavy)
    const ForceCtx x = force_ctx(a, i);
    ForceAcc f = {};
    // Two neighbours per iteration (the row's masks expanded in order, the particle itself skipped), so a warp runs
    // half as many iterations as its lane with the most neighbours; the next entry is fetched as soon as the
    // current one is decoded.
    const uint2* row = nl.ent + (size_t)i * nl.maxe;
    uint2 next = cnt > 0u ? __ldg(row) : make_uint2(0u, 0u);
    uint32_t k = 1, first = 0, mask = 0;
    float shx = 0.0f, shy = 0.0f, shz = 0.0f;
    auto pull = [&](uint32_t& j, float& sx, float& sy, float& sz) -> bool {
        for (;;) {
            if (mask == 0u) {
                if (k > cnt) return false;
                decode_entry(a.grid, next.x, first, shx, shy, shz);
                mask = next.y;
                if (k < cnt) next = __ldg(row + k);
                k++;
            }
            j = first + (uint32_t)(__ffs(mask) - 1);
            mask &= mask - 1u;
            sx = shx;
            sy = shy;
            sz = shz;
            if (j != i) return true;
        }
    };
    const bool periodic = a.grid.periodic;
    for (;;) {
        uint32_t j1, j2;
        float s1x, s1y, s1z, s2x, s2y, s2z;
        if (!pull(j1, s1x, s1y, s1z)) break;
        if (!pull(j2, s2x, s2y, s2z)) {
            force_term<kMorris, kSigma>(a, x, j1, s1x, s1y, s1z, f);
            break;
        }
        if (periodic)
            force_pair<kMorris, true, kSigma, true>(a, x, j1, s1x, s1y, s1z, j2, s2x, s2y, s2z, f);
        else
            force_pair<kMorris, false, kSigma, true>(a, x, j1, s1x, s1y, s1z, j2, s2x, s2y, s2z, f);
    }
    const uint32_t bn = nl.bcnt[i];
    if (bn == kBoundaryWalk)
        boundary_forces<1>(a, b, i, x, f, 0);
    else if (bn != 0u)
        boundary_forces_rows(a, b, i, x, f, row + cnt, bn);
    finish_force(a, i, x, f);
}

template <bool kMorris, bool kSigma>
__global__ void __launch_bounds__(128, 7) k_forces(StepArgs a, CellsDev c, BoundaryDev b, NbrDev nl) {
    forces_ordinary<kMorris, kSigma>(a, c, b, nl, blockIdx.x * blockDim.x + threadIdx.x);
}

// Forces of one heavy particle (force-queue particle i) by one warp.
template <bool kMorris>
__device__ __forceinline__ void forces_heavy_item(const StepArgs& a, const CellsDev& c, const BoundaryDev& b,
                                                  const NbrDev& nl, const uint32_t i, const int lane) {
    {
        const ForceCtx x = force_ctx(a, i);
        ForceAcc f = {};
        const uint32_t cnt = nl.cnt[i];
        if (cnt != kHeavyMark && (cnt & kPooled) != 0u) {
            // the lane's accepted blocks, kept by k_density_heavy in this lane's visiting order
            const size_t base = (size_t)(cnt & ~kPooled) * 32 + lane;
            const uint32_t kept = nl.pool_cnt[base];
            const uint2* seg = nl.pool + base * kPoolLaneEntries;
            for (uint32_t e = 0; e < kept; ++e) {
                uint32_t first, mask;
                float shx, shy, shz;
                row_entry(a.grid, seg[e], first, mask, shx, shy, shz);
                while (mask != 0u) {
                    const uint32_t j = first + (uint32_t)(__ffs(mask) - 1);
                    mask &= mask - 1u;
                    if (j != i) force_term<kMorris>(a, x, j, shx, shy, shz, f);
                }
            }
        } else {
            for_each_subcell_lane(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], x.pi.x, x.pi.y, x.pi.z,
                                  x.hi + x.hi, 0.0f, lane,
                                  [&](uint32_t jb, uint32_t je, float shx, float shy, float shz) {
                                      for (uint32_t j = jb; j < je; ++j) {
                                          if (j == i) continue;
                                          force_term<kMorris>(a, x, j, shx, shy, shz, f);
                                      }
                                  });
        }
        if (b.n != 0) boundary_forces<32>(a, b, i, x, f, lane);
#pragma unroll
        for (int q = 0; q < 3; q++) {
            f.ap[q] = warp_sum_butterfly(f.ap[q]);
            f.av[q] = warp_sum_butterfly(f.av[q]);
            f.as[q] = warp_sum_butterfly(f.as[q]);
            f.bp[q] = warp_sum_butterfly(f.bp[q]);
            f.bf[q] = warp_sum_butterfly(f.bf[q]);
        }
        if (lane == 0) finish_force(a, i, x, f);
    }
}

// Forces of the heavy particles: one warp per particle.
template <bool kMorris>
__global__ void __launch_bounds__(128, 2) k_forces_heavy(StepArgs a, CellsDev c, BoundaryDev b, NbrDev nl) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nh = *nl.fheavy_n;
    for (uint32_t w = warp; w < nh; w += nwarps) forces_heavy_item<kMorris>(a, c, b, nl, nl.fheavy[w], lane);
}

// Particles with long rows (kRowHeavy < cnt <= maxe): one warp per particle, row entry e on lane e mod 32, each
// lane expanding its entries' masks in order; lane sums combined by the butterfly.

__device__ __forceinline__ void density_row_item(const StepArgs& a, const BoundaryDev& b, const NbrDev& nl,
                                                 const uint32_t i, const int lane) {
    {
        const float4 pi = a.ph[i];
        const uint32_t cnt = nl.cnt[i];
        const uint2* row = nl.ent + (size_t)i * nl.maxe;
        float rho = 0.0f;
        for (uint32_t e = lane; e < cnt; e += 32) {
            uint32_t first, mask;
            float shx, shy, shz;
            row_entry(a.grid, row[e], first, mask, shx, shy, shz);
            while (mask != 0u) {
                const uint32_t j = first + (uint32_t)(__ffs(mask) - 1);
                mask &= mask - 1u;
                density_term(a, pi, j, shx, shy, shz, rho);
            }
        }
        rho = warp_sum_butterfly(rho);
        float rb = 0.0f;
        if (b.n != 0) rb = warp_sum_butterfly(boundary_density<32>(a, b, i, pi, lane));
        if (lane == 0) {
            const float rh = rho + rb;
            if (!isfinite(rh)) atomicOr(a.err, 0x2u);
            const float pt = pressure_term(rh, a.phys.rho0, a.phys.B);
            a.rp[i] = make_float2(rh, pt);
            const float4 ki = a.kc[i];
            a.fr[i] = make_float4(rh, pt, ki.x, ki.z);
            nl.frow[atomicAdd(nl.frow_n, 1u)] = i;
        }
    }
}

__global__ void __launch_bounds__(128, 4) k_density_row(StepArgs a, BoundaryDev b, NbrDev nl) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nq = *nl.drow_n;
    for (uint32_t w = warp; w < nq; w += nwarps) density_row_item(a, b, nl, nl.drow[w], lane);
}

template <bool kMorris>
__device__ __forceinline__ void forces_row_item(const StepArgs& a, const BoundaryDev& b, const NbrDev& nl,
                                                const uint32_t i, const int lane) {
    {
        const ForceCtx x = force_ctx(a, i);
        const uint32_t cnt = nl.cnt[i];
        const uint2* row = nl.ent + (size_t)i * nl.maxe;
        ForceAcc f = {};
        for (uint32_t e = lane; e < cnt; e += 32) {
            uint32_t first, mask;
            float shx, shy, shz;
            row_entry(a.grid, row[e], first, mask, shx, shy, shz);
            while (mask != 0u) {
                const uint32_t j = first + (uint32_t)(__ffs(mask) - 1);
                mask &= mask - 1u;
                if (j != i) force_term<kMorris>(a, x, j, shx, shy, shz, f);
            }
        }
        if (b.n != 0) boundary_forces<32>(a, b, i, x, f, lane);
#pragma unroll
        for (int q = 0; q < 3; q++) {
            f.ap[q] = warp_sum_butterfly(f.ap[q]);
            f.av[q] = warp_sum_butterfly(f.av[q]);
            f.as[q] = warp_sum_butterfly(f.as[q]);
            f.bp[q] = warp_sum_butterfly(f.bp[q]);
            f.bf[q] = warp_sum_butterfly(f.bf[q]);
        }
        if (lane == 0) finish_force(a, i, x, f);
    }
}

template <bool kMorris>
__global__ void __launch_bounds__(128, 4) k_forces_row(StepArgs a, BoundaryDev b, NbrDev nl) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nq = *nl.frow_n;
    for (uint32_t w = warp; w < nq; w += nwarps) forces_row_item<kMorris>(a, b, nl, nl.frow[w], lane);
}

// ------------------------------------------------------------------ segmented (multi-scene) passes
static_assert(sizeof(SegLaunch) <= 32000, "segmented launch table must fit the kernel parameter space");

// Scene of work item `it`: the last k with item_start[k] <= it (uniform over the CTA).
__device__ __forceinline__ uint32_t seg_scene_of(const SegLaunch& L, uint32_t it) {
    uint32_t lo = 0, hi = L.nscenes - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (L.item_start[mid] <= it)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Persistent loop of the ordinary segmented kernels: CTA b takes `chunk` consecutive work items at a time, turn by
// turn (items b*chunk .., then (b + gridDim.x)*chunk .., the queue walked round robin, items scene by scene);
// body(scene, i) for every particle slot of an item. The item, and so
// the scene, follows from blockIdx alone, which keeps the scene's argument blocks warp-uniform: the compiler reads
// them into uniform registers as it does a kernel's own arguments.
template <class Body>
__device__ __forceinline__ void seg_items(const SegLaunch& L, Body&& body) {
    for (uint32_t base = blockIdx.x * L.chunk; base < L.total_items; base += gridDim.x * L.chunk) {
        const uint32_t end = base + L.chunk < L.total_items ? base + L.chunk : L.total_items;
        for (uint32_t it = base; it < end; ++it) {
            const uint32_t k = seg_scene_of(L, it);
            body(L.sc[k], (it - L.item_start[k]) * kSegItem + threadIdx.x);
        }
    }
}

// Loop of the warp segmented kernels over the scenes: body(scene).
template <class Body>
__device__ __forceinline__ void seg_scenes(const SegLaunch& L, Body&& body) {
    for (uint32_t k = 0; k < L.nscenes; ++k) body(L.sc[k]);
}

template <bool kPeriodic>
__global__ void __launch_bounds__(128, 7) k_density_seg(const __grid_constant__ SegLaunch L) {
    seg_items(L, [&](const SegScene& S, uint32_t i) { density_ordinary<kPeriodic>(S.a, S.c, S.b, S.nl, i); });
}

template <bool kMorris, bool kSigma>
__global__ void __launch_bounds__(128, 6) k_forces_seg(const __grid_constant__ SegLaunch L) {
    seg_items(L, [&](const SegScene& S, uint32_t i) { forces_ordinary<kMorris, kSigma>(S.a, S.c, S.b, S.nl, i); });
}

// Warp kernels: every warp strides over scene 0's queue, then scene 1's, and so on.
__global__ void __launch_bounds__(128, 2) k_density_heavy_seg(const __grid_constant__ SegLaunch L, int overflow) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    seg_scenes(L, [&](const SegScene& S) {
        const uint32_t* q = overflow ? S.nl.dover : S.nl.heavy;
        const uint32_t nh = *(overflow ? S.nl.dover_n : S.nl.heavy_n);
        for (uint32_t w = warp; w < nh; w += nwarps) density_heavy_item(S.a, S.c, S.b, S.nl, w, q[w], !overflow, lane);
    });
}

__global__ void __launch_bounds__(128, 4) k_density_row_seg(const __grid_constant__ SegLaunch L) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    seg_scenes(L, [&](const SegScene& S) {
        const uint32_t nq = *S.nl.drow_n;
        for (uint32_t w = warp; w < nq; w += nwarps) density_row_item(S.a, S.b, S.nl, S.nl.drow[w], lane);
    });
}

template <bool kMorris>
__global__ void __launch_bounds__(128, 2) k_forces_heavy_seg(const __grid_constant__ SegLaunch L) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    seg_scenes(L, [&](const SegScene& S) {
        const uint32_t nh = *S.nl.fheavy_n;
        for (uint32_t w = warp; w < nh; w += nwarps) forces_heavy_item<kMorris>(S.a, S.c, S.b, S.nl, S.nl.fheavy[w], lane);
    });
}

template <bool kMorris>
__global__ void __launch_bounds__(128, 4) k_forces_row_seg(const __grid_constant__ SegLaunch L) {
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    seg_scenes(L, [&](const SegScene& S) {
        const uint32_t nq = *S.nl.frow_n;
        for (uint32_t w = warp; w < nq; w += nwarps) forces_row_item<kMorris>(S.a, S.b, S.nl, S.nl.frow[w], lane);
    });
}

// The ordinary and the box-heavy kernels of a pass are independent of each other (the heavy queue is filled by the
// reorder kernel), so the host runs them on two streams; the overflow queue is filled by k_density and summed
// after it on its stream.
// A launch of 256-thread blocks with a launch priority (kept by graph capture, unlike the stream's).
template <class... Exp, class... Act>
cudaError_t launch_with_priority(void (*kernel)(Exp...), uint32_t blocks, cudaStream_t stream, int priority,
                                 Act&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * blocks);
    cfg.blockDim = dim3(128);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = priority;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Act>(args)...);
}

cudaError_t launch_density(DensityKernel kind, uint32_t blocks, cudaStream_t stream, int priority, StepArgs a,
                           CellsDev c, BoundaryDev b, NbrDev nl) {
    if (kind == kDensityHeavy)
        return launch_with_priority(k_density_heavy, blocks, stream, priority, a, c, b, nl, (const uint32_t*)nl.heavy,
                                    (const uint32_t*)nl.heavy_n, true);
    if (kind == kDensityOverflow)
        k_density_heavy<<<2 * blocks, 128, 0, stream>>>(a, c, b, nl, nl.dover, nl.dover_n, false);
    else if (kind == kDensityRow)
        k_density_row<<<2 * blocks, 128, 0, stream>>>(a, b, nl);
    else if (a.grid.periodic)  // blocks of 128 threads at 72 registers: 28 warps per SM without spills
        k_density<true><<<2 * blocks, 128, 0, stream>>>(a, c, b, nl);
    else
        k_density<false><<<2 * blocks, 128, 0, stream>>>(a, c, b, nl);
    return cudaGetLastError();
}

cudaError_t launch_forces(ForceKernel kind, bool morris, uint32_t blocks, cudaStream_t stream, int priority, StepArgs a,
                          CellsDev c, BoundaryDev b, NbrDev nl) {
    if (kind == kForcesHeavy) {
        if (morris) return launch_with_priority(k_forces_heavy<true>, blocks, stream, priority, a, c, b, nl);
        return launch_with_priority(k_forces_heavy<false>, blocks, stream, priority, a, c, b, nl);
    }
    if (kind == kForcesRow) {
        if (morris)
            k_forces_row<true><<<2 * blocks, 128, 0, stream>>>(a, b, nl);
        else
            k_forces_row<false><<<2 * blocks, 128, 0, stream>>>(a, b, nl);
    } else {
        // the cohesion term is compiled out when the surface tension constant is zero (the reference's configs);
        // blocks of 128 threads at 72 registers keep 28 warps per SM resident (blocks of 256 would allow 24)
        const bool sigma = a.phys.sigma_on != 0;
        if (morris && sigma)
            k_forces<true, true><<<2 * blocks, 128, 0, stream>>>(a, c, b, nl);
        else if (morris)
            k_forces<true, false><<<2 * blocks, 128, 0, stream>>>(a, c, b, nl);
        else if (sigma)
            k_forces<false, true><<<2 * blocks, 128, 0, stream>>>(a, c, b, nl);
        else
            k_forces<false, false><<<2 * blocks, 128, 0, stream>>>(a, c, b, nl);
    }
    return cudaGetLastError();
}

// Per-particle neighbour counts (sumAllNeighbors, cuda/src/algorithm/Algorithm.cu:234-268).
cudaError_t launch_segmented(SegPass pass, const SegLaunch& L, uint32_t ctas, cudaStream_t stream, int priority,
                             bool periodic, bool morris, bool sigma) {
    if (L.nscenes == 0) return cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(128);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = priority;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    switch (pass) {
        case kSegDensity:
            return periodic ? cudaLaunchKernelEx(&cfg, k_density_seg<true>, L) : cudaLaunchKernelEx(&cfg, k_density_seg<false>, L);
        case kSegDensityHeavy:
            return cudaLaunchKernelEx(&cfg, k_density_heavy_seg, L, 0);
        case kSegDensityOverflow:
            return cudaLaunchKernelEx(&cfg, k_density_heavy_seg, L, 1);
        case kSegDensityRow:
            return cudaLaunchKernelEx(&cfg, k_density_row_seg, L);
        case kSegForces:
            if (morris)
                return sigma ? cudaLaunchKernelEx(&cfg, k_forces_seg<true, true>, L)
                             : cudaLaunchKernelEx(&cfg, k_forces_seg<true, false>, L);
            return sigma ? cudaLaunchKernelEx(&cfg, k_forces_seg<false, true>, L)
                         : cudaLaunchKernelEx(&cfg, k_forces_seg<false, false>, L);
        case kSegForcesHeavy:
            return morris ? cudaLaunchKernelEx(&cfg, k_forces_heavy_seg<true>, L)
                          : cudaLaunchKernelEx(&cfg, k_forces_heavy_seg<false>, L);
        case kSegForcesRow:
            return morris ? cudaLaunchKernelEx(&cfg, k_forces_row_seg<true>, L)
                          : cudaLaunchKernelEx(&cfg, k_forces_row_seg<false>, L);
    }
    return cudaErrorInvalidValue;
}

__global__ void __launch_bounds__(256, 4) k_neighbor_counts(StepArgs a, CellsDev c, uint32_t* counts,
                                                         unsigned long long* total) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = 0;
    if (i < a.n) {
        const float4 pi = a.ph[i];
        const bool periodic = a.grid.periodic;
        fluid_candidates<true>(a, c, pi, [&](uint32_t jb, uint32_t je, float shx, float shy, float shz) {
            for (uint32_t j = jb; j < je; ++j) {
                if (j == i) continue;
                const float4 pj = __ldg(a.ph + j);
                const float xj = periodic ? pj.x + shx : pj.x;
                const float yj = periodic ? pj.y + shy : pj.y;
                const float zj = periodic ? pj.z + shz : pj.z;
                const float dx = xj - pi.x, dy = yj - pi.y, dz = zj - pi.z;
                const float r2 = dist2(dx, dy, dz);
                const float twoh = pj.w + pj.w;
                if (r2 <= twoh * twoh) cnt++;
            }
        });
        if (counts) counts[i] = cnt;
    }
    __shared__ unsigned long long s[8];
    unsigned long long v = cnt;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
        atomicAdd(total, t);
    }
}

}  // namespace asph
