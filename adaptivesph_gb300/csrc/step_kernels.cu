// step_kernels.cu — the per-step kernels of the particle pipeline (plain step: SphSimulation::update,
// cuda/src/simulation/SphSimulation.cu:101-120).
//
// Layout in HBM (structure of arrays, one entry per particle, cell-sorted after every step):
//   ph  float4 (x, y, z, h)       vm  float4 (vx, vy, vz, m)     acc float4 (ax, ay, az, 0)
//   kc  float4 (1/h, coef/h^3, dcoef/h^4, m)   rp float2 (rho, p/rho^2)   rad float   id uint32
// One thread per particle; neighbour loops visit the candidate cells in the canonical order of
// asph_device.cuh and accumulate sequentially, so every sum has a fixed, reproducible order.
#include "asph_device.cuh"
#include "asph_kernels.cuh"

namespace asph {

__device__ __forceinline__ void kick(float& vx, float& vy, float& vz, float ax, float ay, float az, float hdt,
                                     float maxv) {
    // halfKickVelocities (cuda/src/algorithm/Algorithm.cu:270-284)
    vx = fmaf(ax, hdt, vx);
    vy = fmaf(ay, hdt, vy);
    vz = fmaf(az, hdt, vz);
    const float len = sqrtf(fmaf(vz, vz, fmaf(vy, vy, vx * vx)));
    if (len > maxv) {
        const float s = maxv / len;
        vx = vx * s;
        vy = vy * s;
        vz = vz * s;
    }
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u < v ? u : v;
    }
    return v;
}

// Two smallest values of the warp (a < b; ~0 when absent), merged into the global pair (S, T):
// old = atomicMin(S, a); T <- min(T, max(old, a), b). Every value but the global minimum is offered to T.
__device__ __forceinline__ void top2_merge(uint64_t v, unsigned long long* S, unsigned long long* T) {
    const uint64_t a = warp_min_u64(v);
    const uint64_t second = warp_min_u64(v == a ? ~0ull : v);
    if ((threadIdx.x & 31) == 0 && a != ~0ull) {
        const uint64_t old = atomicMin(S, (unsigned long long)a);
        const uint64_t lost = old > a ? old : a;
        atomicMin(T, (unsigned long long)lost);
        if (second != ~0ull) atomicMin(T, (unsigned long long)second);
    }
}

// Closing half-kick of the previous step (when pending), opening half-kick, drift with the domain clamp
// (updatePositions, Algorithm.cu:286-298), then the cell key of the new position (assignParticlesToCells,
// cuda/src/algorithm/neighbors/NeighborKernels.cu:5-15) and the two smallest (reference cell, slot) pairs
// that decide the reference's cell-boundary quirk (NeighborKernels.cu:17-44).
__global__ void __launch_bounds__(256) k_integrate_keys(StepArgs a, float dt, float pending_half, int has_pending,
                                                        uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                        unsigned long long* q3) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = a.n;
    uint64_t q = ~0ull;
    if (i < n) {
        float4 ph = a.ph[i];
        float4 vm = a.vm[i];
        const float4 ac = a.acc[i];
        const float half = dt / 2.0f;
        if (has_pending) kick(vm.x, vm.y, vm.z, ac.x, ac.y, ac.z, pending_half, a.phys.max_velocity);
        kick(vm.x, vm.y, vm.z, ac.x, ac.y, ac.z, half, a.phys.max_velocity);
        float x[3] = {fmaf(vm.x, dt, ph.x), fmaf(vm.y, dt, ph.y), fmaf(vm.z, dt, ph.z)};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (!a.grid.periodic) {
                x[c] = x[c] < a.grid.dmin[c] ? a.grid.dmin[c] : x[c];
                x[c] = x[c] > a.grid.dmax[c] ? a.grid.dmax[c] : x[c];
            } else {
                if (x[c] < a.grid.dmin[c]) x[c] = x[c] + a.grid.scale[c];
                else if (x[c] >= a.grid.dmax[c]) x[c] = x[c] - a.grid.scale[c];
            }
        }
        ph.x = x[0];
        ph.y = x[1];
        ph.z = x[2];
        a.ph[i] = ph;
        a.vm[i] = vm;
        uint32_t key, refkey;
        cell_of(a.grid, x[0], x[1], x[2], key, refkey);
        keys[i] = key;
        vals[i] = i;
        q = ((uint64_t)refkey << 32) | a.id[i];
    }
    if (q3 != nullptr) top2_merge(q, q3, q3 + 1);
}

// Keys of the current positions without moving anything (grid rebuild for diagnostics).
__global__ void __launch_bounds__(256) k_keys(StepArgs a, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                              unsigned long long* q3) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t q = ~0ull;
    if (i < a.n) {
        const float4 ph = a.ph[i];
        uint32_t key, refkey;
        cell_of(a.grid, ph.x, ph.y, ph.z, key, refkey);
        keys[i] = key;
        vals[i] = i;
        q = ((uint64_t)refkey << 32) | a.id[i];
    }
    if (q3 != nullptr) top2_merge(q, q3, q3 + 1);
}

// Boundary keys; the reference slot of a boundary particle is its index in the caller's array.
__global__ void __launch_bounds__(256) k_boundary_keys(GridDev g, const float4* __restrict__ pos, uint32_t n,
                                                       uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                       unsigned long long* q3) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t q = ~0ull;
    if (i < n) {
        const float4 p = pos[i];
        uint32_t key, refkey;
        cell_of(g, p.x, p.y, p.z, key, refkey);
        keys[i] = key;
        vals[i] = i;
        q = ((uint64_t)refkey << 32) | i;
    }
    top2_merge(q, q3, q3 + 1);
}

// Excluded reference cells from the two smallest (cell, slot) pairs: cells of sorted slots 0 and 1 when they
// differ; the only cell when there is one particle.
__global__ void k_excluded(const unsigned long long* q3, const uint32_t* n_ptr, uint32_t n_host, uint32_t* ex,
                           int periodic) {
    const uint32_t n = n_ptr ? *n_ptr : n_host;
    uint32_t e0 = kNone, e1 = kNone;
    if (!periodic && n > 0) {
        const uint64_t S = q3[0], T = q3[1];
        if (n == 1) {
            e0 = (uint32_t)(S >> 32);
        } else if ((S >> 32) != (T >> 32)) {
            e0 = (uint32_t)(S >> 32);
            e1 = (uint32_t)(T >> 32);
        }
    }
    ex[0] = e0;
    ex[1] = e1;
}

// Gathers every particle array into cell-sorted order, forms the kernel constants, and fills the sub-cell
// tables (start, end, max h) and the global max h.
__global__ void __launch_bounds__(256) k_reorder_cells(StepArgs a, ReorderArgs r) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = a.n;
    if (k >= n) return;
    const uint32_t src = r.vals_sorted[k];
    const uint32_t key = r.keys_sorted[k];
    const float4 ph = r.ph_in[src];
    const float4 vm = r.vm_in[src];
    a.ph[k] = ph;
    a.vm[k] = vm;
    a.acc[k] = r.acc_in[src];
    a.rad[k] = r.rad_in[src];
    a.id[k] = r.id_in[src];
    if (r.rp_in != nullptr) a.rp[k] = r.rp_in[src];
    float invh, wc, dwc;
    kernel_consts(ph.w, invh, wc, dwc);
    a.kc[k] = make_float4(invh, wc, dwc, vm.w);
    const uint32_t lin = lin_of_key(a.grid, key);
    if (k == 0 || r.keys_sorted[k - 1] != key) r.start[lin] = k;
    if (k + 1 == n || r.keys_sorted[k + 1] != key) r.end[lin] = k + 1;
    // max h of the cell: one atomic per run of equal keys within the warp
    const unsigned peers = __match_any_sync(__activemask(), key);
    float hm = ph.w;
    for (unsigned m = peers; m; m &= m - 1) {
        const float o = __shfl_sync(peers, ph.w, __ffs(m) - 1);
        hm = o > hm ? o : hm;
    }
    if ((threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1)) {
        atomicMax(reinterpret_cast<int*>(r.hmax) + lin, __float_as_int(hm));
        const uint32_t sx = compact1by2(key), sy = compact1by2(key >> 1), sz = compact1by2(key >> 2);
        const uint32_t rk = (sx >> 1) + (uint32_t)a.grid.gs[0] * ((sy >> 1) + (uint32_t)a.grid.gs[1] * (sz >> 1));
        atomicMax(reinterpret_cast<int*>(r.hmax_ref) + rk, __float_as_int(hm));
    }
}

// Rebuilds the sub-cell tables from cell-sorted keys in place (after a stable compaction).
__global__ void __launch_bounds__(256) k_cells_only(GridDev g, const uint32_t* __restrict__ keys, const uint32_t* n_ptr,
                                                    uint32_t* start, uint32_t* end) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *n_ptr;
    if (k >= n) return;
    const uint32_t key = keys[k];
    const uint32_t lin = lin_of_key(g, key);
    if (k == 0 || keys[k - 1] != key) start[lin] = k;
    if (k + 1 == n || keys[k + 1] != key) end[lin] = k + 1;
}

__global__ void __launch_bounds__(256) k_boundary_reorder(GridDev g, const float4* __restrict__ pos_in,
                                                          const float* __restrict__ psi_in, float friction,
                                                          const uint32_t* __restrict__ keys_sorted,
                                                          const uint32_t* __restrict__ vals_sorted, uint32_t n,
                                                          float4* pos_out, float* fric_out, uint32_t* start,
                                                          uint32_t* end, uint8_t* refflag) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t src = vals_sorted[k];
    const uint32_t key = keys_sorted[k];
    float4 p = pos_in[src];
    p.w = psi_in[src];
    pos_out[k] = p;
    fric_out[k] = friction;
    const uint32_t lin = lin_of_key(g, key);
    if (k == 0 || keys_sorted[k - 1] != key) start[lin] = k;
    if (k + 1 == n || keys_sorted[k + 1] != key) end[lin] = k + 1;
    const uint32_t sx = compact1by2(key), sy = compact1by2(key >> 1), sz = compact1by2(key >> 2);
    refflag[(sx >> 1) + (uint32_t)g.gs[0] * ((sy >> 1) + (uint32_t)g.gs[1] * (sz >> 1))] = 1;
}

// True when any reference cell of the query box of p holds boundary particles.
__device__ __forceinline__ bool boundary_near(const GridDev& g, const BoundaryDev& b, float px, float py, float pz,
                                              float R) {
    if (b.n == 0) return false;
    int32_t lo[3], hi[3];
    const float p[3] = {px, py, pz};
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; a++) ok &= box_axis(g, a, p[a], R, lo[a], hi[a]);
    if (!ok) return false;
    for (int32_t z = lo[2] >> 1; z <= (hi[2] >> 1); z++)
        for (int32_t y = lo[1] >> 1; y <= (hi[1] >> 1); y++)
            for (int32_t x = lo[0] >> 1; x <= (hi[0] >> 1); x++) {
                int32_t cx = x, cy = y, cz = z;
                if (g.periodic) {
                    cx = (cx % g.gs[0] + g.gs[0]) % g.gs[0];
                    cy = (cy % g.gs[1] + g.gs[1]) % g.gs[1];
                    cz = (cz % g.gs[2] + g.gs[2]) % g.gs[2];
                }
                if (__ldg(b.refflag + cx + g.gs[0] * (cy + g.gs[1] * cz))) return true;
            }
    return false;
}

// Periodic image of a listed neighbour: the index keeps 27 bits, the cell's image offset (-1, 0, +1 per axis)
// is packed into the top 5 bits.
constexpr uint32_t kIdxBits = 27;
constexpr uint32_t kIdxMask = (1u << kIdxBits) - 1u;

__device__ __forceinline__ uint32_t shift_code(const GridDev& g, float shx, float shy, float shz) {
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

// Fluid density term of neighbour j (computeDensities, cuda/src/algorithm/Algorithm.cu:17-54); returns false when j
// fails the support test r^2 <= (2 h_j)^2.
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

// The candidate cells of the density/force passes: reference cells of [x - 2h_i, x + 2h_i].
template <class Body>
__device__ __forceinline__ void fluid_candidates(const StepArgs& a, const CellsDev& c, float4 pi, Body&& body) {
    const float R = pi.w + pi.w;
    for_each_cell<true>(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], pi.x, pi.y, pi.z, R, 0.0f, body);
}

// computeDensities (cuda/src/algorithm/Algorithm.cu:17-54) + computeBoundaryDensityContribution
// (cuda/src/algorithm/BoundaryAlgorithm.cu:15-51), then p/rho^2 for the force pass. The scan also records the
// accepted neighbours (self included) in the particle's list, in candidate order, for the force pass.
__global__ void __launch_bounds__(256, 3) k_density(StepArgs a, CellsDev c, BoundaryDev b, NbrDev nl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 pi = a.ph[i];
    const bool periodic = a.grid.periodic;
    uint32_t cnt = 0;
    uint32_t* col = nl.idx + i;
    const uint32_t stride = nl.stride, maxn = nl.maxn;
    float rho = 0.0f;
    fluid_candidates(a, c, pi, [&](uint32_t jb, uint32_t je, float shx, float shy, float shz) {
        const uint32_t code = periodic ? (shift_code(a.grid, shx, shy, shz) << kIdxBits) : 0u;
        for (uint32_t j = jb; j < je; ++j) {
            if (!density_term(a, pi, j, shx, shy, shz, rho)) continue;
            if (cnt < maxn) col[(size_t)cnt * stride] = j | code;
            cnt++;
        }
    });
    nl.cnt[i] = cnt;
    const float R = pi.w + pi.w;
    float rb = 0.0f;
    if (boundary_near(a.grid, b, pi.x, pi.y, pi.z, R)) {
        const float4 ki = a.kc[i];
        const float cut = R * R;
        for_each_cell<false>(a.grid, b.start, b.end, nullptr, nullptr, b.ex0, b.ex1, pi.x, pi.y, pi.z, R, 0.0f,
                             [&](uint32_t kb, uint32_t ke, float shx, float shy, float shz) {
                                 for (uint32_t k = kb; k < ke; ++k) {
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
    }
    const float rh = rho + rb;
    if (!isfinite(rh)) atomicOr(a.err, 0x2u);
    a.rp[i] = make_float2(rh, pressure_term(rh, a.phys.rho0, a.phys.B));
}

// Per-particle constants and accumulators of the force pass.
struct ForceAcc {
    float apx, apy, apz, avx, avy, avz, asx, asy, asz;
};

// Pressure, viscosity and cohesion terms of fluid neighbour j (cuda/src/algorithm/Algorithm.cu:56-221).
template <bool kMorris>
__device__ __forceinline__ void force_term(const StepArgs& a, float4 pi, float4 vi, float rhoi, float pti, float Ki,
                                           float ei, bool visc_on, bool sigma_on, uint32_t j, float shx, float shy,
                                           float shz, ForceAcc& f) {
    const bool periodic = a.grid.periodic;
    const float4 pj = __ldg(a.ph + j);
    const float xj = periodic ? pj.x + shx : pj.x;
    const float yj = periodic ? pj.y + shy : pj.y;
    const float zj = periodic ? pj.z + shz : pj.z;
    const float dx = pi.x - xj, dy = pi.y - yj, dz = pi.z - zj;
    const float r2 = dist2(dx, dy, dz);
    const float twoh = pj.w + pj.w;
    if (r2 > twoh * twoh) return;
    const float4 kj = __ldg(a.kc + j);
    const float2 rpj = __ldg(a.rp + j);
    const float r = sqrtf(r2);
    float ux, uy, uz;
    if (r > 0.0f) {
        const float ir = 1.0f / r;
        ux = dx * ir;
        uy = dy * ir;
        uz = dz * ir;
    } else {
        ux = 0.0f;
        uy = 1.0f;
        uz = 0.0f;
    }
    const float dw = kernel_dw(r, kj.x, kj.z);
    const float mj = kj.w;
    {
        const float sp = (mj * dw) * (pti + rpj.y);
        f.apx = fmaf(-sp, ux, f.apx);
        f.apy = fmaf(-sp, uy, f.apy);
        f.apz = fmaf(-sp, uz, f.apz);
    }
    if (visc_on) {
        const float4 vj = __ldg(a.vm + j);
        const float vdx = vi.x - vj.x, vdy = vi.y - vj.y, vdz = vi.z - vj.z;
        const float rhoj = rpj.x;
        if (!kMorris) {
            const float comp = fmaf(vdz, dz, fmaf(vdy, dy, vdx * dx));
            if (comp < 0.0f) {
                const float nuij = Ki / (rhoi + rhoj);
                const float piv = (-nuij * comp) / (r2 + ei);
                const float sv = (mj * piv) * dw;
                f.avx = fmaf(-sv, ux, f.avx);
                f.avy = fmaf(-sv, uy, f.avy);
                f.avz = fmaf(-sv, uz, f.avz);
            }
        } else {
            const float coef = ((mj * a.phys.nu) * (rhoi + rhoj)) / (rhoi * rhoj);
            const float sv = coef * ((r * dw) / (r2 + ei));
            f.avx = fmaf(sv, vdx, f.avx);
            f.avy = fmaf(sv, vdy, f.avy);
            f.avz = fmaf(sv, vdz, f.avz);
        }
    }
    if (sigma_on) {
        const float ss = mj * kernel_w(r, kj.x, kj.y);
        f.asx = fmaf(ss, ux, f.asx);
        f.asy = fmaf(ss, uy, f.asy);
        f.asz = fmaf(ss, uz, f.asz);
    }
}

// computeExternalAccelerations, computePressureAccelerations, computeViscosityAccelerations,
// computeSurfaceTensionAccelerations (cuda/src/algorithm/Algorithm.cu:56-232) and
// computeBoundaryPressureAcceleration / computeBoundaryFrictionAcceleration
// (cuda/src/algorithm/BoundaryAlgorithm.cu:53-162) in one pass over the neighbour list; each term keeps its own
// accumulator and they are added to gravity in the reference's kernel order.
template <bool kMorris>
__global__ void __launch_bounds__(256, 3) k_forces(StepArgs a, CellsDev c, BoundaryDev b, NbrDev nl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 pi = a.ph[i];
    const float4 vi = a.vm[i];
    const float2 rpi = a.rp[i];
    const float hi = pi.w, mi = vi.w, rhoi = rpi.x, pti = rpi.y;
    const float c0 = a.phys.c0;
    const float Ki = ((2.0f * a.phys.alpha) * hi) * c0;
    const float ei = (0.01f * hi) * hi;
    const float R = hi + hi;
    const bool visc_on = a.phys.visc_on, sigma_on = a.phys.sigma_on, periodic = a.grid.periodic;
    ForceAcc f = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const uint32_t cnt = nl.cnt[i];
    if (cnt <= nl.maxn) {
        const uint32_t* col = nl.idx + i;
        for (uint32_t k = 0; k < cnt; ++k) {
            uint32_t j;
            float shx, shy, shz;
            decode_entry(a.grid, __ldg(col + (size_t)k * nl.stride), j, shx, shy, shz);
            if (j == i) continue;
            force_term<kMorris>(a, pi, vi, rhoi, pti, Ki, ei, visc_on, sigma_on, j, shx, shy, shz, f);
        }
    } else {
        fluid_candidates(a, c, pi, [&](uint32_t jb, uint32_t je, float shx, float shy, float shz) {
            for (uint32_t j = jb; j < je; ++j) {
                if (j == i) continue;
                force_term<kMorris>(a, pi, vi, rhoi, pti, Ki, ei, visc_on, sigma_on, j, shx, shy, shz, f);
            }
        });
    }
    float bpx = 0.f, bpy = 0.f, bpz = 0.f, bfx = 0.f, bfy = 0.f, bfz = 0.f;
    if (boundary_near(a.grid, b, pi.x, pi.y, pi.z, R)) {
        const float4 ki = a.kc[i];
        const float cut = R * R;
        for_each_cell<false>(a.grid, b.start, b.end, nullptr, nullptr, b.ex0, b.ex1, pi.x, pi.y, pi.z, R, 0.0f,
                             [&](uint32_t kb, uint32_t ke, float shx, float shy, float shz) {
                                 for (uint32_t k = kb; k < ke; ++k) {
                                     const float4 pb = __ldg(b.pos + k);
                                     const float xb = periodic ? pb.x + shx : pb.x;
                                     const float yb = periodic ? pb.y + shy : pb.y;
                                     const float zb = periodic ? pb.z + shz : pb.z;
                                     const float dx = pi.x - xb, dy = pi.y - yb, dz = pi.z - zb;
                                     const float r2 = dist2(dx, dy, dz);
                                     if (r2 > cut) continue;
                                     const float r = sqrtf(r2);
                                     float ux, uy, uz;
                                     if (r > 0.0f) {
                                         const float ir = 1.0f / r;
                                         ux = dx * ir;
                                         uy = dy * ir;
                                         uz = dz * ir;
                                     } else {
                                         ux = 0.0f;
                                         uy = 1.0f;
                                         uz = 0.0f;
                                     }
                                     const float dw = kernel_dw(r, ki.x, ki.z);
                                     const float psi = pb.w;
                                     const float sp = (psi * pti) * dw;
                                     bpx = fmaf(-sp, ux, bpx);
                                     bpy = fmaf(-sp, uy, bpy);
                                     bpz = fmaf(-sp, uz, bpz);
                                     const float comp = fmaf(vi.z, dz, fmaf(vi.y, dy, vi.x * dx));
                                     if (comp < 0.0f) {
                                         const float nub = ((__ldg(b.fric + k) * hi) * c0) / (2.0f * rhoi);
                                         const float pib = (-nub * comp) / (r2 + ei);
                                         const float sf = (psi * pib) * dw;
                                         bfx = fmaf(-sf, ux, bfx);
                                         bfy = fmaf(-sf, uy, bfy);
                                         bfz = fmaf(-sf, uz, bfz);
                                     }
                                 }
                             });
    }
    float ax = a.phys.gravity[0], ay = a.phys.gravity[1], az = a.phys.gravity[2];
    ax = ax + f.apx;
    ay = ay + f.apy;
    az = az + f.apz;
    if (visc_on) {
        ax = ax + f.avx;
        ay = ay + f.avy;
        az = az + f.avz;
    }
    if (sigma_on) {
        const float fs = a.phys.sigma / mi;
        ax = ax + fs * f.asx;
        ay = ay + fs * f.asy;
        az = az + fs * f.asz;
    }
    ax = ax + bpx;
    ay = ay + bpy;
    az = az + bpz;
    ax = ax + bfx;
    ay = ay + bfy;
    az = az + bfz;
    if (!(isfinite(ax) && isfinite(ay) && isfinite(az))) atomicOr(a.err, 0x2u);
    a.acc[i] = make_float4(ax, ay, az, 0.0f);
}

cudaError_t launch_forces(bool morris, uint32_t blocks, cudaStream_t stream, StepArgs a, CellsDev c, BoundaryDev b,
                          NbrDev nl) {
    if (morris)
        k_forces<true><<<blocks, 256, 0, stream>>>(a, c, b, nl);
    else
        k_forces<false><<<blocks, 256, 0, stream>>>(a, c, b, nl);
    return cudaGetLastError();
}

// Per-particle neighbour counts (sumAllNeighbors, cuda/src/algorithm/Algorithm.cu:234-268).
__global__ void __launch_bounds__(256) k_neighbor_counts(StepArgs a, CellsDev c, uint32_t* counts,
                                                         unsigned long long* total) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = 0;
    if (i < a.n) {
        const float4 pi = a.ph[i];
        const float R = pi.w + pi.w;
        const bool periodic = a.grid.periodic;
        for_each_cell<true>(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], pi.x, pi.y, pi.z, R, 0.0f,
                            [&](uint32_t jb, uint32_t je, float shx, float shy, float shz) {
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
    // block sum then one atomic
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

// Export: positions (w = 0), velocities with the pending closing half-kick, densities, radii.
__global__ void __launch_bounds__(256) k_export(StepArgs a, float pending_half, int has_pending, float4* pos_out,
                                                float4* vel_out, float* rho_out, float* rad_out, uint32_t* id_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 ph = a.ph[i];
    float4 vm = a.vm[i];
    if (pos_out) pos_out[i] = make_float4(ph.x, ph.y, ph.z, 0.0f);
    if (vel_out) {
        if (has_pending) {
            const float4 ac = a.acc[i];
            kick(vm.x, vm.y, vm.z, ac.x, ac.y, ac.z, pending_half, a.phys.max_velocity);
        }
        vel_out[i] = make_float4(vm.x, vm.y, vm.z, 0.0f);
    }
    if (rho_out) rho_out[i] = a.rp[i].x;
    if (rad_out) rad_out[i] = a.rad[i];
    if (id_out) id_out[i] = a.id[i];
}

// FP64 totals (mass, momentum, kinetic energy, volume) and min_i h_i / (c0 + |v_i|) for the CFL step.
__global__ void __launch_bounds__(256) k_totals(StepArgs a, float pending_half, int has_pending, double* out,
                                                unsigned int* cfl_min_bits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[6] = {0, 0, 0, 0, 0, 0};
    float cfl = 3.402823466e38f;
    if (i < a.n) {
        const float4 ph = a.ph[i];
        float4 vm = a.vm[i];
        if (has_pending) {
            const float4 ac = a.acc[i];
            kick(vm.x, vm.y, vm.z, ac.x, ac.y, ac.z, pending_half, a.phys.max_velocity);
        }
        const double m = vm.w;
        v[0] = m;
        v[1] = m * vm.x;
        v[2] = m * vm.y;
        v[3] = m * vm.z;
        v[4] = 0.5 * m * ((double)vm.x * vm.x + (double)vm.y * vm.y + (double)vm.z * vm.z);
        const float rho = a.rp[i].x;
        v[5] = rho > 0.0f ? m / (double)rho : 0.0;
        const float speed = sqrtf(fmaf(vm.z, vm.z, fmaf(vm.y, vm.y, vm.x * vm.x)));
        cfl = ph.w / (a.phys.c0 + speed);
    }
    __shared__ double s[8][6];
    __shared__ float sc[8];
#pragma unroll
    for (int k = 0; k < 6; k++) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        v[k] = t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cfl = fminf(cfl, __shfl_xor_sync(0xffffffffu, cfl, o));
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 6; k++) s[threadIdx.x >> 5][k] = v[k];
        sc[threadIdx.x >> 5] = cfl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            for (int k = 0; k < 6; k++) s[0][k] += s[w][k];
            sc[0] = fminf(sc[0], sc[w]);
        }
        for (int k = 0; k < 6; k++) atomicAdd(out + k, s[0][k]);
        if (cfl_min_bits) atomicMin(cfl_min_bits, __float_as_uint(sc[0]));
    }
}

// getDensityInfo (cuda/src/simulation/SphSimulation.cu:249-285); the mean is accumulated in FP64.
__global__ void __launch_bounds__(256) k_density_info(StepArgs a, float threshold, float rest, double* sum,
                                                      unsigned int* minmax, unsigned int* counts) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float d = a.rp[i].x;
    const float ratio = d / rest - 1.0f;
    atomicAdd(sum, (double)d);
    // order-preserving integer image of the float for min/max
    const uint32_t u = __float_as_uint(d);
    const uint32_t s = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    atomicMin(minmax, s);
    atomicMax(minmax + 1, s);
    if (ratio < -threshold) atomicAdd(counts, 1u);
    if (ratio >= -threshold && ratio <= threshold) atomicAdd(counts + 1, 1u);
    if (ratio > threshold) atomicAdd(counts + 2, 1u);
}

}  // namespace asph
