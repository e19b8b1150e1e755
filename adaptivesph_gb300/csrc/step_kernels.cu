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
// old = atomicMin(S, a); T <- min(T, max(old, a), b). Every value but the global minimum is offered to T. T only
// decreases and the values are distinct, so a value not below the T the warp reads can be neither of the final
// two: such warps skip the atomics (most of them, once the first warps have run).
__device__ __forceinline__ void top2_merge(uint64_t v, unsigned long long* S, unsigned long long* T) {
    const uint64_t a = warp_min_u64(v);
    const uint64_t second = warp_min_u64(v == a ? ~0ull : v);
    if ((threadIdx.x & 31) == 0 && a != ~0ull) {
        const uint64_t t_now = *reinterpret_cast<volatile unsigned long long*>(T);
        if (a < t_now) {
            const uint64_t old = atomicMin(S, (unsigned long long)a);
            const uint64_t lost = old > a ? old : a;
            atomicMin(T, (unsigned long long)lost);
            if (second < t_now) atomicMin(T, (unsigned long long)second);
        }
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
    const uint32_t n = count_of(a);
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
    if (i < count_of(a)) {
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
    const uint32_t n = count_of(a);
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
    const float twoh = ph.w + ph.w;
    a.pq[k] = make_float4(ph.x, ph.y, ph.z, twoh * twoh);
    if (r.heavy != nullptr && box_cells(a.grid, ph, ph.w + ph.w) > kHeavyCells) r.heavy[atomicAdd(r.heavy_n, 1u)] = k;
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

// Fixed-order reductions. A grid of kRedBlocks blocks strides over the particles (the thread that handles particle i
// depends only on i), every block reduces its threads in a fixed tree and writes one row of kRedCols partials, and
// k_reduce_rows adds the rows in a fixed order: the results are bit-identical from run to run, which FP64 atomics
// across blocks would not be.
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();  // sh may still be read from the previous column
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = sh[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    return t;
}

__device__ __forceinline__ double block_min(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = sh[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) t = fmin(t, sh[w]);
    return t;
}

// FP64 totals (mass, momentum, kinetic energy, volume; columns 0-5) and min_i h_i / (c0 + |v_i|) for the CFL step
// (column 6), one row of partials per block.
__global__ void __launch_bounds__(256) k_totals(StepArgs a, float pending_half, int has_pending, double* rows) {
    double v[7] = {0, 0, 0, 0, 0, 0, 1.0e300};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const float4 ph = a.ph[i];
        float4 vm = a.vm[i];
        if (has_pending) {
            const float4 ac = a.acc[i];
            kick(vm.x, vm.y, vm.z, ac.x, ac.y, ac.z, pending_half, a.phys.max_velocity);
        }
        const double m = vm.w;
        v[0] += m;
        v[1] += m * vm.x;
        v[2] += m * vm.y;
        v[3] += m * vm.z;
        v[4] += 0.5 * m * ((double)vm.x * vm.x + (double)vm.y * vm.y + (double)vm.z * vm.z);
        const float rho = a.rp[i].x;
        v[5] += rho > 0.0f ? m / (double)rho : 0.0;
        const float speed = sqrtf(fmaf(vm.z, vm.z, fmaf(vm.y, vm.y, vm.x * vm.x)));
        v[6] = fmin(v[6], (double)(ph.w / (a.phys.c0 + speed)));
    }
    __shared__ double sh[8];
    double* row = rows + (size_t)blockIdx.x * kRedCols;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        const double t = block_sum(v[k], sh);
        if (threadIdx.x == 0) row[k] = t;
    }
    const double t = block_min(v[6], sh);
    if (threadIdx.x == 0) row[6] = t;
}

// getDensityInfo (cuda/src/simulation/SphSimulation.cu:249-285): sum of densities (FP64), min, max, and the
// under / normal / over counts (columns 0-5), one row of partials per block.
__global__ void __launch_bounds__(256) k_density_info(StepArgs a, float threshold, float rest, double* rows) {
    double v[6] = {0, 1.0e300, -1.0e300, 0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const float d = a.rp[i].x;
        const float ratio = d / rest - 1.0f;
        v[0] += (double)d;
        v[1] = fmin(v[1], (double)d);
        v[2] = fmax(v[2], (double)d);
        if (ratio < -threshold) v[3] += 1.0;
        if (ratio >= -threshold && ratio <= threshold) v[4] += 1.0;
        if (ratio > threshold) v[5] += 1.0;
    }
    __shared__ double sh[8];
    double* row = rows + (size_t)blockIdx.x * kRedCols;
    double t = block_sum(v[0], sh);
    if (threadIdx.x == 0) row[0] = t;
    t = block_min(v[1], sh);
    if (threadIdx.x == 0) row[1] = t;
    t = -block_min(-v[2], sh);
    if (threadIdx.x == 0) row[2] = t;
    for (int k = 3; k < 6; k++) {
        t = block_sum(v[k], sh);
        if (threadIdx.x == 0) row[k] = t;
    }
}

// out[k] = the sum (or, for the columns in min_mask / max_mask, the min / max) of column k over `nrows` rows,
// added in a fixed order. One block of 256 threads.
__global__ void __launch_bounds__(256) k_reduce_rows(const double* rows, uint32_t nrows, uint32_t ncols,
                                                     uint32_t min_mask, uint32_t max_mask, double* out) {
    __shared__ double sh[8];
    for (uint32_t k = 0; k < ncols; k++) {
        const bool is_min = (min_mask >> k) & 1u, is_max = (max_mask >> k) & 1u;
        double v = is_min ? 1.0e300 : (is_max ? -1.0e300 : 0.0);
        for (uint32_t r = threadIdx.x; r < nrows; r += blockDim.x) {
            const double x = rows[(size_t)r * kRedCols + k];
            v = is_min ? fmin(v, x) : (is_max ? fmax(v, x) : v + x);
        }
        const double t = is_min ? block_min(v, sh) : (is_max ? -block_min(-v, sh) : block_sum(v, sh));
        if (threadIdx.x == 0) out[k] = t;
    }
}

}  // namespace asph
