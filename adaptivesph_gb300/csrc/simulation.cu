// simulation.cu — the host runtime behind the C ABI (include/asph.h): one simulation = device-resident
// particle state + the per-step kernel sequence on one CUDA stream.
//
// Replaces SphSimulation / AdaptiveSphSimulation (cuda/src/simulation/SphSimulation.cu,
// cuda/src/simulation/AdaptiveSphSimulation.cu), NeighborGrid (cuda/src/simulation/neighbors/NeighborGrid.cu),
// ImportedParticleMemory (cuda/src/memory/ImportedParticleMemory.cu) and StaticBoundaryDomain
// (cuda/src/simulation/physics/StaticBoundaryDomain.cu) behind the reference's interface.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <chrono>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/asph.h"
#include "asph_kernels.cuh"
#include "asph_refine.cuh"
#include "batch_internal.h"
#include "boundary_internal.h"

using namespace asph;

// ------------------------------------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

static asph_status fail(asph_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

static asph_status cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return ASPH_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return ASPH_ERR_NO_DEVICE;
    return ASPH_ERR_CUDA;
}

namespace asph {
asph_status report_error(asph_status s, const std::string& msg) { return fail(s, msg); }
asph_status report_cuda_error(cudaError_t e, const char* what) { return cuda_fail(e, what); }
}  // namespace asph

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);        \
    } while (0)

// Drops a stale, non-sticky error left by an earlier runtime call (of this library or of the caller), so that
// the launch checks below report only errors of the launch itself. Sticky errors persist and are still caught.
#define API_ENTRY() (void)cudaGetLastError()

#define CK_LAUNCH(what)                                            \
    do {                                                           \
        cudaError_t e_ = cudaGetLastError();                       \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);         \
    } while (0)

static inline uint32_t blocks_for(uint32_t n, uint32_t t = 256) { return n == 0 ? 1u : (n + t - 1) / t; }

// blocks of 8 warps for the heavy-particle kernels (one warp per heavy particle, grid-stride over the queue)
static constexpr uint32_t kHeavyBlocks = 304;  // grid of the one-warp-per-particle kernels at 600k particles and more

// The grid of the one-warp-per-particle kernels (heavy boxes, overflowed and long rows): they stride over a queue
// whose length is known only on the device, usually a small fraction of the particles, so small simulations get a
// small grid (an empty queue still costs every block of the launch).
uint32_t heavy_blocks(uint32_t n) {
    const uint32_t b = n / 2048u;
    return b < 16u ? 16u : (b > kHeavyBlocks ? kHeavyBlocks : b);
}

// bytes of the per-simulation reduction scratch (totals, CFL minimum, density info)
// reduction scratch: 8 result doubles, then kRedBlocks rows of kRedCols partials (k_totals, k_density_info)
static constexpr size_t kRedBytes = 64 + sizeof(double) * kRedBlocks * kRedCols;

// ------------------------------------------------------------------------------------------------ memory
struct asph_memory {
    void* ptr = nullptr;
    size_t size = 0;
    cudaExternalMemory_t ext = nullptr;
};

// ------------------------------------------------------------------------------------------------ state kernels
namespace {

// Unpacks the SoA state into the reference's separate arrays.
__global__ void k_read_state(StepArgs a, float4* pos, float4* vel, float4* acc, float* rho, float* rad, float* h,
                             float* m, uint32_t* id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 ph = a.ph[i];
    const float4 vm = a.vm[i];
    pos[i] = make_float4(ph.x, ph.y, ph.z, 0.0f);
    vel[i] = make_float4(vm.x, vm.y, vm.z, 0.0f);
    acc[i] = a.acc[i];
    rho[i] = a.rp[i].x;
    rad[i] = a.rad[i];
    h[i] = ph.w;
    m[i] = vm.w;
    id[i] = a.id[i];
}

__global__ void k_write_state(StepArgs a, const float4* pos, const float4* vel, const float4* acc, const float* rho,
                              const float* rad, const float* h, const float* m, const uint32_t* id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 p = pos[i];
    const float4 v = vel[i];
    a.ph[i] = make_float4(p.x, p.y, p.z, h[i]);
    a.vm[i] = make_float4(v.x, v.y, v.z, m[i]);
    const float4 ac = acc[i];
    a.acc[i] = make_float4(ac.x, ac.y, ac.z, 0.0f);
    a.rp[i] = make_float2(rho[i], 0.0f);
    a.rad[i] = rad[i];
    a.id[i] = id[i];
}

// Initial state as the reference's constructor writes it (SphSimulation.cu:29-80): v = 0, a = (g, 0),
// r = r0, h = h0, m = m0; the id is the array slot.
__global__ void k_init_state(StepArgs a, const float4* pos, float r0, float h0, float m0) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float4 p = pos[i];
    a.ph[i] = make_float4(p.x, p.y, p.z, h0);
    a.vm[i] = make_float4(0.0f, 0.0f, 0.0f, m0);
    a.acc[i] = make_float4(a.phys.gravity[0], a.phys.gravity[1], a.phys.gravity[2], 0.0f);
    a.rp[i] = make_float2(0.0f, 0.0f);
    a.rad[i] = r0;
    a.id[i] = i;
}

// Boundary records as the caller passes them (asph_boundary_particle: x, y, z, w, psi; 20 bytes, 4-byte aligned)
// split into the positions and psi that the boundary setup sorts.
__global__ void k_boundary_records(const float* rec, uint32_t nb, float4* pos, float* psi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    const float* r = rec + 5 * (size_t)i;
    pos[i] = make_float4(r[0], r[1], r[2], r[3]);
    psi[i] = r[4];
}

}  // namespace

// ------------------------------------------------------------------------------------------------ simulation
struct BufferSet {
    float4* ph = nullptr;
    float4* vm = nullptr;
    float4* acc = nullptr;
    float2* rp = nullptr;
    float* rad = nullptr;
    uint32_t* id = nullptr;
};

struct asph_simulation {
    asph_parameters P{};
    asph_refinement_parameters R{};
    bool adaptive = false;
    GridDev grid{};
    PhysDev phys{};
    uint32_t cap = 0, n = 0;
    uint32_t bcap = 0, nb = 0;
    uint32_t tpb = 256;

    BufferSet set[2];
    int cur = 0;
    float4* kc = nullptr;
    float4* pq = nullptr;  // [cap] x, y, z, (2h)^2 of the current step (StepArgs::pq)
    float4* fr = nullptr;  // [cap] rho, p/rho^2, 1/h, dcoef/h^4 of the current step (StepArgs::fr)
    uint2* nbr_ent = nullptr;     // [kListEntries * rows_cap] neighbour lists, one row per particle
    uint32_t rows_cap = 0;        // particles the rows are allocated for (grown on demand, never above cap)
    uint8_t* arena = nullptr;     // one allocation holding the fixed-size buffers (carve_fixed)
    uint32_t* nbr_cnt = nullptr;  // [cap]
    uint32_t* nbr_bcnt = nullptr;  // [cap] wall entries of ordinary rows
    uint32_t* heavy_idx = nullptr;  // [cap] queue of heavy particles of the current step
    uint32_t* heavy_n = nullptr;
    uint32_t* fheavy_idx = nullptr;  // [cap] queue of the force pass's warp kernel
    uint32_t* fheavy_n = nullptr;  // [4]: lengths of the fheavy, dover, drow and frow queues
    uint32_t* dover_idx = nullptr;  // [cap] particles whose list row overflowed in the density pass
    uint32_t* drow_idx = nullptr;   // [cap] particles with long rows, density pass
    uint32_t* frow_idx = nullptr;   // [cap] particles with long rows, force pass
    uint2* pool = nullptr;          // [pool_slots * 32 * kPoolLaneEntries] accepted blocks of heavy particles
    uint32_t* pool_cnt = nullptr;   // [pool_slots * 32]
    uint32_t pool_slots = 0;        // capacity / 128, clamped to [64, kPoolSlots]
    uint32_t* keys = nullptr;
    uint32_t* vals = nullptr;
    void* sort_mem = nullptr;
    SortScratch ss{};
    uint32_t* cell_start = nullptr;  // the five sub-cell tables (start, end, max h; the boundary's start, end)
    uint32_t* cell_end = nullptr;    // are carved from one allocation, cell_block
    float* cell_hmax = nullptr;
    uint8_t* cell_block = nullptr;
    uint32_t cells_alloc = 0;
    float* hmax_ref = nullptr;  // [gs.x * gs.y * gs.z] max h per reference cell
    uint32_t refcells_alloc = 0;
    uint32_t* ex = nullptr;
    unsigned long long* q3 = nullptr;
    uint32_t* err = nullptr;
    uint32_t* d_count = nullptr;
    uint8_t* red = nullptr;  // [kRedBytes] reduction scratch of totals, CFL and density info (fixed order)
    uint64_t device_bytes = 0;  // device memory held (device_bytes_for at creation)

    // boundary
    float4* bpos = nullptr;
    float* bfric = nullptr;
    uint32_t* bstart = nullptr;
    uint32_t* bend = nullptr;
    uint8_t* brefflag = nullptr;
    uint32_t brefcells = 0;
    uint32_t bex[2] = {kNone, kNone};

    // refinement scratch
    float* score = nullptr;
    uint32_t* cand = nullptr;
    uint32_t* flag = nullptr;
    uint32_t* ctr = nullptr;
    unsigned long long* slot0 = nullptr;
    uint32_t* block_counts = nullptr;
    uint32_t* rkeys = nullptr;    // [2 * cap] cell keys of the step and their compacted copy
    uint32_t* dbg_ids = nullptr;  // [3 * cap] keep / removed / split id lists (when enabled)
    bool record_ids = false;

    // host-side state
    uint32_t frame = 0;
    uint32_t next_id = 0;
    float pending_half = 0.0f;
    bool has_pending = false;
    bool grid_valid = false;
    asph_refinement_report last_report{};
    uint32_t last_pairs_listed = 0, last_splits_listed = 0;

    // export staging (device), grown on demand
    uint8_t* stage = nullptr;
    size_t stage_bytes = 0;

    // pinned host scratch
    uint32_t* h_ctr = nullptr;
    uint64_t* h_small = nullptr;

    // export targets (imported memory)
    asph_fluid_buffers fbuf{};
    bool have_fbuf = false;
    asph_boundary_buffers bbuf{};
    bool have_bbuf = false;

    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t aux = nullptr;  // heavy-particle kernels, forked from and joined back into `stream`
    int heavy_priority = 0;      // the device's highest stream priority, given to the heavy kernels
    cudaEvent_t ev_fork = nullptr, ev_main = nullptr, ev_aux = nullptr;
    cudaStream_t copy = nullptr;  // device-to-host copies of asynchronous exports (created on first use)
    cudaEvent_t ev_export_ready = nullptr, ev_export_done = nullptr;
    bool export_inflight = false;
    cudaEvent_t ev_refine = nullptr;  // end of a refinement pass whose read-back has not been taken yet
    bool refine_pending = false;
    uint64_t launches = 0;

    // timing
    bool timing = false;
    // plain steps of asph_simulation_step_async replayed from captured graphs (created at the first such step)
    asph::SceneGraph* own_graph = nullptr;
    struct Ev {
        cudaEvent_t a, b;
        int cls;
    };
    std::vector<Ev> events;
    std::vector<cudaEvent_t> event_pool;
    double ms[ASPH_KERNEL_COUNT] = {0};
    uint32_t timed[ASPH_KERNEL_COUNT] = {0};

    // set while a step is captured as a graph: kernels read the count from d_count, grids cover grid_n
    bool graph_mode = false;
    uint32_t grid_n = 0;
    // bumped by every call that changes what a captured step holds by value or by pointer (grid, cell and boundary
    // tables, parameters, particle arrays); a batch's cached graphs are recaptured when it changes
    uint64_t generation = 0;
    // unique over the process's simulations (a recycled address never matches an earlier simulation's graphs)
    uint64_t serial = 0;
    uint32_t span() const { return graph_mode ? grid_n : n; }

    StepArgs args(int s) const {
        StepArgs a;
        a.grid = grid;
        a.phys = phys;
        a.n = span();
        a.np = graph_mode ? d_count : nullptr;
        a.ph = set[s].ph;
        a.vm = set[s].vm;
        a.acc = set[s].acc;
        a.rp = set[s].rp;
        a.rad = set[s].rad;
        a.id = set[s].id;
        a.kc = kc;
        a.err = err;
        a.pq = pq;
        a.fr = fr;
        return a;
    }

    CellsDev cells() const { return CellsDev{cell_start, cell_end, cell_hmax, hmax_ref, ex}; }

    NbrDev nbrs() const {
        return NbrDev{nbr_ent,      nbr_cnt,  heavy_idx,    heavy_n,  fheavy_idx,   fheavy_n,
                      dover_idx,    fheavy_n + 1, drow_idx, fheavy_n + 2, frow_idx, fheavy_n + 3,
                      nbr_bcnt,     pool,     pool_cnt,     pool_slots,   kListEntries, rows_cap};
    }

    BoundaryDev boundary() const {
        return BoundaryDev{bpos, bfric, bstart, bend, brefflag, bex[0], bex[1], nb};
    }

    cudaEvent_t take_event() {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    int tic() {
        if (!timing) return -1;
        Ev ev{take_event(), take_event(), 0};
        cudaEventRecord(ev.a, stream);
        events.push_back(ev);
        return (int)events.size() - 1;
    }
    void toc(int h, int cls) {
        if (h < 0) return;
        events[h].cls = cls;
        cudaEventRecord(events[h].b, stream);
    }
    cudaError_t harvest() {
        cudaError_t first = cudaSuccess;
        for (auto& e : events) {
            float t = 0.f;
            const cudaError_t r = cudaEventElapsedTime(&t, e.a, e.b);
            if (r == cudaSuccess) {
                ms[e.cls] += t;
                timed[e.cls] += 1;
            } else if (first == cudaSuccess) {
                first = r;
            }
            event_pool.push_back(e.a);
            event_pool.push_back(e.b);
        }
        events.clear();
        (void)cudaGetLastError();  // a failed elapsed-time query must not surface in a later launch check
        return first;
    }
};

namespace {

template <class T>
asph_status dalloc(T*& p, size_t count) {
    p = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * count));
    return ASPH_OK;
}

void dfree(void* p) {
    if (p) cudaFree(p);
}

// Device memory a simulation can hold: the sizes asph_simulation_create allocates, with the neighbour rows at the
// capacity (they start smaller and grow; the export staging buffer, allocated on the first export, and the optional
// id lists are not included).
uint64_t device_bytes_for(uint32_t C, uint32_t sort_items, uint32_t ncells, uint32_t refcells, uint32_t nb,
                          bool adaptive) {
    const uint64_t c = C;
    uint64_t b = 0;
    b += 2 * c * (sizeof(float4) * 3 + sizeof(float2) + sizeof(float) + sizeof(uint32_t));  // two buffer sets
    b += c * sizeof(float4) * 3;                          // kernel constants, support operands, force operands
    b += c * kListEntries * sizeof(uint2) + c * sizeof(uint32_t) * 2;                      // rows and counts
    b += c * sizeof(uint32_t) * 5 + sizeof(uint32_t) * 5;                                   // queues
    const uint64_t slots = std::min<uint32_t>(kPoolSlots, std::max<uint32_t>(64u, C / 128u));
    b += slots * 32 * (kPoolLaneEntries * sizeof(uint2) + sizeof(uint32_t));                // heavy pool
    b += (uint64_t)sort_items * sizeof(uint32_t) * 2 + sort_scratch_bytes(sort_items);      // sort
    b += sizeof(uint32_t) * 4 + sizeof(unsigned long long) * 2 + sizeof(uint32_t) * 3 + kRedBytes;
    b += (uint64_t)refcells * (sizeof(float) + 1) + (uint64_t)ncells * sizeof(uint32_t) * 5;  // cell tables
    b += (uint64_t)nb * (sizeof(float4) + sizeof(float));                                  // boundary
    if (adaptive) b += c * sizeof(uint32_t) * 5 + sizeof(uint32_t) * (kCtrNum + 2 + blocks_for(C)) + 8;
    return b;
}

asph_status make_grid(const asph_parameters& P, GridDev& g) {
    std::memset(&g, 0, sizeof(g));
    const float cw = (2.0f * P.base_smoothing_radius) * 2.0f;
    int32_t mx = 1;
    uint64_t ncells = 1;
    float maxscale = 0.0f;
    for (int a = 0; a < 3; a++) {
        g.dmin[a] = P.domain.min[a];
        g.dmax[a] = P.domain.max[a];
        g.scale[a] = P.domain.max[a] - P.domain.min[a];
        if (!(g.scale[a] > 0.0f)) return fail(ASPH_ERR_INVALID_ARGUMENT, "domain max must exceed min on every axis");
        const float q = std::ceil(g.scale[a] / cw);
        if (!(q < 512.5f)) return fail(ASPH_ERR_UNSUPPORTED, "domain spans more than 512 cells of 4 h0 on an axis");
        int32_t gs = (int32_t)q;
        if (gs < 1) gs = 1;
        if (P.boundary_mode == ASPH_BOUNDARY_PERIODIC && gs < 3)
            return fail(ASPH_ERR_UNSUPPORTED, "a periodic box needs at least 3 cells of 4 h0 per axis");
        g.gs[a] = gs;
        g.cs[a] = g.scale[a] / (float)gs;
        g.w[a] = g.cs[a] * 0.5f;
        g.sgs[a] = 2 * gs;
        mx = std::max(mx, g.sgs[a]);
        ncells *= (uint64_t)g.sgs[a];
        maxscale = std::max(maxscale, g.scale[a]);
    }
    uint32_t bits = 1;
    while ((1 << bits) < mx) bits++;
    g.bits = bits;
    g.ncells = (uint32_t)ncells;
    g.periodic = P.boundary_mode == ASPH_BOUNDARY_PERIODIC ? 1 : 0;
    g.cull_margin = 1.0e-5f * maxscale;
    return ASPH_OK;
}

void make_phys(const asph_parameters& P, PhysDev& ph) {
    for (int a = 0; a < 3; a++) ph.gravity[a] = P.gravity[a];
    ph.c0 = P.speed_of_sound;
    ph.rho0 = P.rest_density;
    ph.alpha = P.viscosity_constant;
    ph.sigma = P.surface_tension_constant;
    ph.max_velocity = P.max_velocity;
    ph.h0 = P.base_smoothing_radius;
    ph.r0 = P.base_particle_radius;
    ph.m0 = P.base_particle_mass;
    ph.nu = P.kinematic_viscosity;
    ph.B = ((P.rest_density * P.speed_of_sound) * P.speed_of_sound) / 5.0f;
    ph.morris = P.viscosity_model == ASPH_VISCOSITY_MORRIS ? 1 : 0;
    ph.visc_on = ph.morris ? (P.kinematic_viscosity != 0.0f) : (P.viscosity_constant != 0.0f);
    ph.sigma_on = P.surface_tension_constant != 0.0f;
}

asph_status alloc_cells(asph_simulation* s) {
    const uint32_t refcells = (uint32_t)(s->grid.gs[0] * s->grid.gs[1] * s->grid.gs[2]);
    if (refcells > s->refcells_alloc) {
        dfree(s->hmax_ref);
        s->refcells_alloc = 0;
        asph_status st0 = dalloc(s->hmax_ref, refcells);
        if (st0 != ASPH_OK) return st0;
        s->refcells_alloc = refcells;
    }
    if (s->grid.ncells <= s->cells_alloc) return ASPH_OK;
    dfree(s->cell_block);
    s->cell_block = nullptr;
    s->cell_start = s->cell_end = s->bstart = s->bend = nullptr;
    s->cell_hmax = nullptr;
    s->cells_alloc = 0;
    // one allocation for the five tables (each cudaMalloc costs tens of microseconds at creation)
    const size_t table = ((size_t)s->grid.ncells * sizeof(uint32_t) + 255) / 256 * 256;
    asph_status st;
    if ((st = dalloc(s->cell_block, 5 * table)) != ASPH_OK) return st;
    s->cell_start = reinterpret_cast<uint32_t*>(s->cell_block);
    s->cell_end = reinterpret_cast<uint32_t*>(s->cell_block + table);
    s->cell_hmax = reinterpret_cast<float*>(s->cell_block + 2 * table);
    s->bstart = reinterpret_cast<uint32_t*>(s->cell_block + 3 * table);
    s->bend = reinterpret_cast<uint32_t*>(s->cell_block + 4 * table);
    s->cells_alloc = s->grid.ncells;
    return ASPH_OK;
}

// Sorts the boundary particles (device arrays d_pos / d_psi, nb of them) by sub-cell and builds their tables; also
// writes the caller's imported boundary buffers in the caller's order (initializeBoundaryParticles,
// SphSimulation.cu:287-333).
asph_status setup_boundary_device(asph_simulation* s, const float4* d_pos, const float* d_psi, uint32_t nb) {
    if (nb > s->bcap) {
        dfree(s->bpos);
        dfree(s->bfric);
        s->bcap = 0;
        asph_status st;
        if ((st = dalloc(s->bpos, nb)) != ASPH_OK) return st;
        if ((st = dalloc(s->bfric, nb)) != ASPH_OK) return st;
        s->bcap = nb;
    }
    const uint32_t refcells = (uint32_t)(s->grid.gs[0] * s->grid.gs[1] * s->grid.gs[2]);
    if (refcells > s->brefcells) {
        dfree(s->brefflag);
        s->brefcells = 0;
        asph_status st;
        if ((st = dalloc(s->brefflag, refcells)) != ASPH_OK) return st;
        s->brefcells = refcells;
    }
    s->nb = nb;
    CK(cudaMemsetAsync(s->bstart, 0xff, sizeof(uint32_t) * s->grid.ncells, s->stream));
    CK(cudaMemsetAsync(s->bend, 0, sizeof(uint32_t) * s->grid.ncells, s->stream));
    CK(cudaMemsetAsync(s->brefflag, 0, refcells, s->stream));
    s->bex[0] = s->bex[1] = kNone;
    if (nb == 0) return ASPH_OK;
    CK(cudaMemsetAsync(s->q3, 0xff, 2 * sizeof(unsigned long long), s->stream));
    k_boundary_keys<<<blocks_for(nb), 256, 0, s->stream>>>(s->grid, d_pos, nb, s->keys, s->vals, s->q3);
    CK_LAUNCH("k_boundary_keys");
    // the sort reads its item count from device memory
    s->h_ctr[0] = nb;
    CK(cudaMemcpyAsync(s->d_count + 1, s->h_ctr, sizeof(uint32_t), cudaMemcpyHostToDevice, s->stream));
    s->launches += 1 + radix_sort_pairs(s->keys, s->vals, s->d_count + 1, nb, 3 * s->grid.bits, s->ss, s->err,
                                        s->stream);
    CK_LAUNCH("boundary sort");
    k_excluded<<<1, 1, 0, s->stream>>>(s->q3, nullptr, nb, s->ex + 2, s->grid.periodic);
    k_boundary_reorder<<<blocks_for(nb), 256, 0, s->stream>>>(s->grid, d_pos, d_psi, s->P.domain.friction, s->keys,
                                                              s->vals, nb, s->bpos, s->bfric, s->bstart, s->bend,
                                                              s->brefflag);
    CK_LAUNCH("k_boundary_reorder");
    s->launches += 2;
    CK(cudaMemcpyAsync(s->h_ctr, s->ex + 2, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->bex[0] = s->h_ctr[0];
    s->bex[1] = s->h_ctr[1];
    if (s->have_bbuf) {
        std::vector<float4> colors(nb, make_float4(0.3f, 0.3f, 0.3f, 0.2f));
        std::vector<float> radii(nb, s->P.base_particle_radius);
        const asph_memory* mp = s->bbuf.positions;
        const asph_memory* mr = s->bbuf.radii;
        const asph_memory* mc = s->bbuf.colors;
        if (mp && mp->size >= sizeof(float4) * nb)
            CK(cudaMemcpyAsync(mp->ptr, d_pos, sizeof(float4) * nb, cudaMemcpyDeviceToDevice, s->stream));
        if (mr && mr->size >= sizeof(float) * nb)
            CK(cudaMemcpyAsync(mr->ptr, radii.data(), sizeof(float) * nb, cudaMemcpyHostToDevice, s->stream));
        if (mc && mc->size >= sizeof(float4) * nb)
            CK(cudaMemcpyAsync(mc->ptr, colors.data(), sizeof(float4) * nb, cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return ASPH_OK;
}

// The same from host boundary particles (StaticBoundaryDomain::Particle, position + psi).
// Whether this device's kernels read pageable host memory coherently through the host's page tables (address
// translation over NVLink-C2C, as on Grace-Blackwell): creation then reads the caller's arrays in place, one pass
// at link bandwidth, instead of staging them through a pageable copy. Without translation through the host's page
// tables (pageable access by page migration) the pages would move to the device, so that case copies.
std::atomic<int> g_host_reads_in_place{1};  // asph_debug_host_reads_in_place: 0 forces the staging copies

bool device_reads_host_in_place(const void* p, size_t align) {
    if (g_host_reads_in_place.load(std::memory_order_relaxed) == 0) return false;
    if (reinterpret_cast<uintptr_t>(p) % align != 0) return false;
    int dev = 0, pageable = 0, host_tables = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return pageable == 1 && host_tables == 1;
}

// The caller's boundary records: read in place (device_reads_host_in_place) or copied as they are, then split into
// positions and psi on the device.
// At creation (spare) the other buffer set, not yet used, holds the unsorted positions and psi when they fit.
asph_status setup_boundary(asph_simulation* s, const asph_boundary_particle* b, uint32_t nb, bool spare = false) {
    if (nb == 0) return setup_boundary_device(s, nullptr, nullptr, 0);
    static_assert(sizeof(asph_boundary_particle) == 5 * sizeof(float), "boundary records are 5 floats");
    float4* d_pos = nullptr;
    float* d_psi = nullptr;
    float* d_rec = nullptr;
    const float* rec = reinterpret_cast<const float*>(b);
    const bool own = !(spare && nb <= s->cap);
    asph_status st = ASPH_OK;
    if (own) {
        st = dalloc(d_pos, nb);
        if (st == ASPH_OK) st = dalloc(d_psi, nb);
    } else {
        d_pos = s->set[1 - s->cur].ph;
        d_psi = s->set[1 - s->cur].rad;
    }
    cudaError_t e = cudaSuccess;
    if (st == ASPH_OK && !device_reads_host_in_place(b, alignof(float))) {
        st = dalloc(d_rec, 5 * (size_t)nb);
        if (st == ASPH_OK)
            e = cudaMemcpyAsync(d_rec, b, sizeof(asph_boundary_particle) * nb, cudaMemcpyHostToDevice, s->stream);
        rec = d_rec;
    }
    if (st == ASPH_OK && e == cudaSuccess) {
        k_boundary_records<<<blocks_for(nb), 256, 0, s->stream>>>(rec, nb, d_pos, d_psi);
        e = cudaGetLastError();
        s->launches++;
    }
    if (st == ASPH_OK) st = e == cudaSuccess ? setup_boundary_device(s, d_pos, d_psi, nb) : cuda_fail(e, "boundary upload");
    cudaStreamSynchronize(s->stream);
    dfree(d_rec);
    if (own) {
        dfree(d_pos);
        dfree(d_psi);
    }
    return st;
}

asph_status upload_count(asph_simulation* s) {
    s->h_ctr[0] = s->n;
    CK(cudaMemcpyAsync(s->d_count, s->h_ctr, sizeof(uint32_t), cudaMemcpyHostToDevice, s->stream));
    return ASPH_OK;
}

// Sort the current particles by sub-cell, gather into the other buffer set, build the cell tables.
asph_status build_grid(asph_simulation* s, bool integrate, float dt, bool carry_rho) {
    const uint32_t n = s->span();
    StepArgs a = s->args(s->cur);
    CK(cudaMemsetAsync(s->q3, 0xff, 2 * sizeof(unsigned long long), s->stream));
    int h = s->tic();
    if (integrate) {
        k_integrate_keys<<<blocks_for(n), 256, 0, s->stream>>>(a, dt, s->pending_half, s->has_pending ? 1 : 0,
                                                               s->keys, s->vals, s->q3);
        CK_LAUNCH("k_integrate_keys");
        s->has_pending = false;
    } else {
        k_keys<<<blocks_for(n), 256, 0, s->stream>>>(a, s->keys, s->vals, s->q3);
        CK_LAUNCH("k_keys");
    }
    s->toc(h, ASPH_KERNEL_INTEGRATE);
    s->launches++;
    h = s->tic();
    s->launches += radix_sort_pairs(s->keys, s->vals, s->d_count, n, 3 * s->grid.bits, s->ss, s->err, s->stream);
    CK_LAUNCH("radix sort");
    s->toc(h, ASPH_KERNEL_SORT);
    CK(cudaMemsetAsync(s->cell_start, 0xff, sizeof(uint32_t) * s->grid.ncells, s->stream));
    CK(cudaMemsetAsync(s->cell_end, 0, sizeof(uint32_t) * s->grid.ncells, s->stream));
    CK(cudaMemsetAsync(s->cell_hmax, 0, sizeof(float) * s->grid.ncells, s->stream));
    CK(cudaMemsetAsync(s->hmax_ref, 0, sizeof(float) * s->refcells_alloc, s->stream));
    CK(cudaMemsetAsync(s->heavy_n, 0, sizeof(uint32_t), s->stream));
    k_excluded<<<1, 1, 0, s->stream>>>(s->q3, s->graph_mode ? s->d_count : nullptr, n, s->ex, s->grid.periodic);
    CK_LAUNCH("k_excluded");
    ReorderArgs r;
    r.keys_sorted = s->keys;
    r.vals_sorted = s->vals;
    r.ph_in = s->set[s->cur].ph;
    r.vm_in = s->set[s->cur].vm;
    r.acc_in = s->set[s->cur].acc;
    r.rad_in = s->set[s->cur].rad;
    r.id_in = s->set[s->cur].id;
    r.rp_in = carry_rho ? s->set[s->cur].rp : nullptr;
    r.start = s->cell_start;
    r.end = s->cell_end;
    r.hmax = s->cell_hmax;
    r.hmax_ref = s->hmax_ref;
    r.heavy = s->heavy_idx;
    r.heavy_n = s->heavy_n;
    const int nxt = 1 - s->cur;
    StepArgs b = s->args(nxt);
    h = s->tic();
    k_reorder_cells<<<blocks_for(n), 256, 0, s->stream>>>(b, r);
    CK_LAUNCH("k_reorder_cells");
    s->toc(h, ASPH_KERNEL_REORDER);
    s->launches += 2;
    s->cur = nxt;
    s->grid_valid = true;
    return ASPH_OK;
}

// Rows for n particles and the growth a refinement pass may add before the next allocation check (the grid bound
// a captured step is keyed with: n + n/8 + 256, in multiples of 256), never above the capacity.
uint32_t rows_for(uint32_t n, uint32_t cap) {
    const uint64_t b = ((uint64_t)n + n / 8 + 256 + 255) / 256 * 256;
    return (uint32_t)std::min<uint64_t>(b, std::max<uint32_t>(cap, 1u));
}

// The neighbour rows (128 entries, 1 KB per particle) are allocated for the particles present plus headroom, not
// for the whole capacity (4x the initial count in the adaptive dam break), and grown when a step needs more: rows
// are rebuilt every step, so growing drops nothing. Growing waits for the simulation's streams (the old rows may
// be in use) and bumps the generation, so captured steps holding the old rows are captured again. Never called
// while a step is being captured (the caller grows the rows first).
asph_status ensure_rows(asph_simulation* s, uint32_t need) {
    if (need <= s->rows_cap) return ASPH_OK;
    if (s->graph_mode) return fail(ASPH_ERR_INVALID_ARGUMENT, "neighbour rows must be grown before a capture");
    const uint32_t want = rows_for(need + need / 4, s->cap);
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaStreamSynchronize(s->aux));
    dfree(s->nbr_ent);
    s->nbr_ent = nullptr;
    s->rows_cap = 0;
    asph_status st = dalloc(s->nbr_ent, (size_t)kListEntries * want);
    if (st != ASPH_OK) return st;
    s->rows_cap = want;
    s->generation++;
    return ASPH_OK;
}

// The ordinary kernel of each neighbour pass runs on the simulation's stream, the heavy-particle kernel on the
// auxiliary stream, concurrently:
//   main: k_density ------------(wait heavy density)-- k_forces ------------(wait heavy forces)--
//   aux : (wait reorder) k_density_heavy -- (wait k_density) k_forces_heavy
// The force kernels read the densities of all particles, hence the cross waits; the heavy force queue also holds
// the particles whose neighbour rows overflowed in k_density.
asph_status run_density(asph_simulation* s) {
    StepArgs a = s->args(s->cur);
    int h = s->tic();
    CK(cudaMemsetAsync(s->fheavy_n, 0, 4 * sizeof(uint32_t), s->stream));
    CK(cudaEventRecord(s->ev_fork, s->stream));
    CK(cudaStreamWaitEvent(s->aux, s->ev_fork, 0));
    CK(launch_density(kDensityHeavy, heavy_blocks(s->span()), s->aux, s->heavy_priority, a, s->cells(), s->boundary(), s->nbrs()));
    CK(launch_density(kDensityOrdinary, blocks_for(s->span()), s->stream, 0, a, s->cells(), s->boundary(), s->nbrs()));
    CK(launch_density(kDensityOverflow, heavy_blocks(s->span()), s->stream, 0, a, s->cells(), s->boundary(), s->nbrs()));
    CK(launch_density(kDensityRow, heavy_blocks(s->span()), s->stream, 0, a, s->cells(), s->boundary(), s->nbrs()));
    CK(cudaEventRecord(s->ev_main, s->stream));
    CK(cudaEventRecord(s->ev_aux, s->aux));
    CK(cudaStreamWaitEvent(s->stream, s->ev_aux, 0));
    s->toc(h, ASPH_KERNEL_DENSITY);
    s->launches += 4;
    return ASPH_OK;
}

asph_status run_forces(asph_simulation* s) {
    StepArgs a = s->args(s->cur);
    int h = s->tic();
    CK(cudaStreamWaitEvent(s->aux, s->ev_main, 0));
    CK(launch_forces(kForcesHeavy, s->phys.morris != 0, heavy_blocks(s->span()), s->aux, s->heavy_priority, a, s->cells(), s->boundary(),
                     s->nbrs()));
    CK(launch_forces(kForcesOrdinary, s->phys.morris != 0, blocks_for(s->span()), s->stream, 0, a, s->cells(), s->boundary(),
                     s->nbrs()));
    CK(launch_forces(kForcesRow, s->phys.morris != 0, heavy_blocks(s->span()), s->stream, 0, a, s->cells(), s->boundary(),
                     s->nbrs()));
    CK(cudaEventRecord(s->ev_aux, s->aux));
    CK(cudaStreamWaitEvent(s->stream, s->ev_aux, 0));
    s->toc(h, ASPH_KERNEL_FORCES);
    s->launches += 3;
    return ASPH_OK;
}

RefineArgs refine_args(asph_simulation* s) {
    RefineArgs r;
    r.score = s->score;
    r.cand = s->cand;
    r.flag = s->flag;
    r.ctr = s->ctr;
    r.slot0 = s->slot0;
    r.keep_ids = s->record_ids ? s->dbg_ids : nullptr;
    r.removed_ids = s->record_ids ? s->dbg_ids + s->cap : nullptr;
    r.split_ids = s->record_ids ? s->dbg_ids + 2 * (size_t)s->cap : nullptr;
    r.mqueue = s->dover_idx;  // the density-overflow queue is dead after the force pass
    r.err = s->err;
    const asph_refinement_parameters& R = s->R;
    r.min_mass = R.min_mass_ratio * s->P.base_particle_mass;
    r.max_mass = R.max_mass_ratio * s->P.base_particle_mass;
    r.max_batch_ratio = R.max_batch_ratio;
    r.eps = R.split_epsilon;
    r.alpha = R.split_alpha;
    r.center_ratio = R.split_center_mass_ratio;
    r.vertex_ratio = R.split_vertex_mass_ratio;
    r.vel_split = R.velocity_split_min_speed;
    r.vel_merge = R.velocity_merge_max_speed;
    r.vort_split = R.vorticity_split_min;
    r.vort_merge = R.vorticity_merge_max;
    r.iface_split = R.interface_split_distance_ratio;
    r.iface_merge = R.interface_merge_distance_ratio;
    r.fs_split = R.free_surface_split_deficit;
    r.fs_merge = R.free_surface_merge_deficit;
    r.r0 = s->P.base_particle_radius;
    r.m0 = s->P.base_particle_mass;
    r.rho0 = s->P.rest_density;
    r.criterion = R.criterion;
    return r;
}

uint32_t id_bits(uint32_t next_id) {
    uint32_t b = 1;
    while (b < 32 && (1ull << b) < (uint64_t)next_id) b++;
    return b;
}

// One refinement pass (performAdaptiveRefinement, AdaptiveSphSimulation.cu:102-252), enqueued; its counters are
// read back into h_ctr at the end and taken by refine_finish.
asph_status refine_enqueue(asph_simulation* s) {
    const uint32_t n = s->n;
    s->last_report = asph_refinement_report{};
    s->last_report.frame = s->frame;
    s->last_report.count_before = n;
    s->last_report.count_after = n;
    if (n <= 1) return ASPH_OK;  // identifyAndMergeParticles returns early (AdaptiveSphSimulation.cu:197-200)
    int h = s->tic();
    RefineArgs r = refine_args(s);
    std::memset(s->h_ctr, 0, sizeof(uint32_t) * kCtrNum);
    s->h_ctr[kCtrNextId] = s->next_id;
    CK(cudaMemcpyAsync(s->ctr, s->h_ctr, sizeof(uint32_t) * kCtrNum, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(s->slot0, 0xff, sizeof(unsigned long long), s->stream));
    // criteria that walk neighbours evaluate the split scores on the cells of the compacted set
    const bool walks = s->R.criterion == ASPH_CRITERION_VORTICITY || s->R.criterion == ASPH_CRITERION_FREE_SURFACE;
    if (walks) {
        // keep the cell keys of this step: the selection sorts reuse the sort buffers
        CK(cudaMemcpyAsync(s->rkeys, s->keys, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s->stream));
    }
    StepArgs a = s->args(s->cur);
    const uint32_t nbk = blocks_for(n);
    // merge selection
    int hp = s->tic();
    k_merge_score<<<nbk, 256, 0, s->stream>>>(a, s->cells(), r);
    k_merge_limits<<<1, 1, 0, s->stream>>>(r, n);
    k_select_ids<<<nbk, 256, 0, s->stream>>>(a, s->ctr + kCtrSortN, s->keys, s->vals);
    CK_LAUNCH("merge selection");
    s->launches += 3;
    s->launches += radix_sort_pairs(s->keys, s->vals, s->ctr + kCtrSortN, n, id_bits(s->next_id), s->ss, s->err,
                                    s->stream);
    k_select_scores<<<nbk, 256, 0, s->stream>>>(s->score, s->ctr + kCtrSortN, 0, s->vals, s->keys);
    s->launches += 1 + radix_sort_pairs(s->keys, s->vals, s->ctr + kCtrSortN, n, 32, s->ss, s->err, s->stream);
    s->toc(hp, ASPH_KERNEL_REFINE_MERGE_SELECT);
    // candidates, pairs + merges
    hp = s->tic();
    k_cand_init<<<nbk, 256, 0, s->stream>>>(r, n);
    k_mark_eligible<<<nbk, 256, 0, s->stream>>>(r, s->vals);
    k_merge_candidates<<<nbk, 256, 0, s->stream>>>(a, s->cells(), r);
    k_merge_candidates_heavy<<<heavy_blocks(n), 256, 0, s->stream>>>(a, s->cells(), r);
    k_merge_pairs<<<nbk, 256, 0, s->stream>>>(a, r);
    CK_LAUNCH("merge");
    s->toc(hp, ASPH_KERNEL_REFINE_MERGE);
    // stable compaction into the other buffer set (also carries the cell keys for a split pass that walks cells)
    hp = s->tic();
    k_compact_count<<<nbk, 256, 0, s->stream>>>(s->flag, n, s->block_counts);
    k_compact_scan<<<1, 1024, 0, s->stream>>>(s->block_counts, nbk, n, r);
    const int nxt = 1 - s->cur;
    StepArgs b = s->args(nxt);
    uint32_t* keys_c = s->rkeys + s->cap;
    k_compact_scatter<<<nbk, 256, 0, s->stream>>>(a, b, s->flag, s->block_counts, walks ? s->rkeys : nullptr,
                                                   keys_c);
    CK_LAUNCH("compaction");
    s->launches += 8;
    s->cur = nxt;
    StepArgs c = s->args(s->cur);
    if (walks) {
        // the compacted keys are still cell-sorted: rebuild the tables for the split criterion's search
        CK(cudaMemsetAsync(s->cell_start, 0xff, sizeof(uint32_t) * s->grid.ncells, s->stream));
        CK(cudaMemsetAsync(s->cell_end, 0, sizeof(uint32_t) * s->grid.ncells, s->stream));
        k_cells_only<<<nbk, 256, 0, s->stream>>>(s->grid, keys_c, s->ctr + kCtrCount2, s->cell_start, s->cell_end);
        s->launches++;
    }
    s->toc(hp, ASPH_KERNEL_REFINE_COMPACT);
    // split selection (skipped on the device when nothing was removed)
    hp = s->tic();
    k_split_score<<<nbk, 256, 0, s->stream>>>(c, s->cells(), r);
    k_split_limits<<<1, 1, 0, s->stream>>>(r, s->cap, s->tpb);
    k_select_split_ids<<<nbk, 256, 0, s->stream>>>(c, r, s->keys, s->vals);
    CK_LAUNCH("split selection");
    s->launches += 3;
    s->launches += radix_sort_pairs(s->keys, s->vals, s->ctr + kCtrSortN, n, id_bits(s->next_id), s->ss, s->err,
                                    s->stream);
    k_select_scores<<<nbk, 256, 0, s->stream>>>(s->score, s->ctr + kCtrSortN, 1, s->vals, s->keys);
    s->launches += 1 + radix_sort_pairs(s->keys, s->vals, s->ctr + kCtrSortN, n, 32, s->ss, s->err, s->stream);
    s->toc(hp, ASPH_KERNEL_REFINE_SPLIT_SELECT);
    hp = s->tic();
    k_split_apply<<<nbk, 256, 0, s->stream>>>(c, r, s->vals);
    k_refine_finish<<<1, 1, 0, s->stream>>>(r);
    CK_LAUNCH("split");
    s->launches += 2;
    CK(cudaMemcpyAsync(s->d_count, s->ctr + kCtrCountOut, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->h_ctr, s->ctr, sizeof(uint32_t) * kCtrNum, cudaMemcpyDeviceToHost, s->stream));
    s->toc(hp, ASPH_KERNEL_REFINE_SPLIT);
    s->toc(h, ASPH_KERNEL_REFINE);
    CK(cudaEventRecord(s->ev_refine, s->stream));
    s->refine_pending = true;
    s->grid_valid = false;
    return ASPH_OK;
}

// Waits for the enqueued refinement pass and takes its counters (new count, next id, report).
asph_status refine_finish(asph_simulation* s) {
    if (!s->refine_pending) return ASPH_OK;
    s->refine_pending = false;
    CK(cudaEventSynchronize(s->ev_refine));
    const uint32_t* c2 = s->h_ctr;
    s->n = c2[kCtrCountOut];
    s->next_id = c2[kCtrNextId];
    s->last_report.merge_eligible = c2[kCtrEligible];
    s->last_report.merge_pairs = c2[kCtrPairs];
    s->last_report.removed = c2[kCtrRemoved];
    s->last_report.split_candidates = c2[kCtrSplitCand];
    s->last_report.split_budget = c2[kCtrSplitBudget];
    s->last_report.splits = c2[kCtrSplits];
    s->last_report.count_after = s->n;
    s->last_pairs_listed = c2[kCtrPairs];
    s->last_splits_listed = c2[kCtrSplits];
    return ASPH_OK;
}

asph_status run_refine(asph_simulation* s) {
    asph_status st = refine_enqueue(s);
    if (st != ASPH_OK) return st;
    return refine_finish(s);
}

// Upper bound of the particle count after a refinement pass started from n: merges remove, each split adds 12,
// and splits exceed removed/12 by at most one block's worth (the reference's guard, Q-8); never above capacity.
uint32_t count_after_refine_bound(const asph_simulation* s) {
    const uint64_t b = (uint64_t)s->n + 12ull * (s->tpb > 0 ? s->tpb : 256);
    return (uint32_t)std::min<uint64_t>(b, s->cap);
}

bool refinement_due(const asph_simulation* s) {
    if (!s->adaptive) return false;
    const uint32_t f = s->frame, i0 = s->R.initial_cooldown, cd = s->R.cooldown;
    return f == i0 || (f > i0 && f % cd == 0);
}

// One step up to last_stage. With defer_refine a refinement pass is only enqueued (refine_finish takes its
// read-back later); the host-side count is then stale until refine_finish.
asph_status run_step(asph_simulation* s, float dt, uint32_t last_stage, bool defer_refine = false) {
    if (!(std::isfinite(dt))) return fail(ASPH_ERR_INVALID_ARGUMENT, "delta time must be finite");
    if (s->n == 0) {
        // nothing to integrate; bookkeeping as the reference (kernels with zero threads)
        if (last_stage >= ASPH_STAGE_ALL) {
            s->pending_half = dt / 2.0f;
            s->has_pending = true;
            s->frame++;
        }
        return ASPH_OK;
    }
    asph_status st;
    if (last_stage < ASPH_STAGE_GRID) {
        // integrate only: keys are computed but the state is not reordered
        StepArgs a = s->args(s->cur);
        CK(cudaMemsetAsync(s->q3, 0xff, 2 * sizeof(unsigned long long), s->stream));
        k_integrate_keys<<<blocks_for(s->n), 256, 0, s->stream>>>(a, dt, s->pending_half, s->has_pending ? 1 : 0,
                                                                  s->keys, s->vals, s->q3);
        CK_LAUNCH("k_integrate_keys");
        s->launches++;
        s->has_pending = false;
        s->grid_valid = false;
        return ASPH_OK;
    }
    if (!s->graph_mode && (st = ensure_rows(s, s->span())) != ASPH_OK) return st;
    if ((st = build_grid(s, true, dt, false)) != ASPH_OK) return st;
    if (last_stage < ASPH_STAGE_DENSITY) return ASPH_OK;
    if ((st = run_density(s)) != ASPH_OK) return st;
    if (last_stage < ASPH_STAGE_FORCES) return ASPH_OK;
    if ((st = run_forces(s)) != ASPH_OK) return st;
    if (last_stage < ASPH_STAGE_ALL) return ASPH_OK;
    if (refinement_due(s)) {
        if ((st = defer_refine ? refine_enqueue(s) : run_refine(s)) != ASPH_OK) return st;
    }
    s->pending_half = dt / 2.0f;
    s->has_pending = true;
    s->frame++;
    return ASPH_OK;
}

asph_status check_errors(asph_simulation* s, bool sync) {
    if (sync) CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpy(s->h_ctr, s->err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    const uint32_t e = s->h_ctr[0] & ~0x4u;
    if (e != 0) {
        char buf[128];
        std::snprintf(buf, sizeof(buf), "device error word 0x%x", e);
        return fail(ASPH_ERR_DEVICE_CHECK, buf);
    }
    return ASPH_OK;
}

asph_status ensure_grid(asph_simulation* s) {
    if (s->grid_valid || s->n == 0) return ASPH_OK;
    return build_grid(s, false, 0.0f, true);
}

// Waits for the copies of an asynchronous export still in flight.
asph_status export_settle(asph_simulation* s) {
    if (!s->export_inflight) return ASPH_OK;
    CK(cudaEventSynchronize(s->ev_export_done));
    s->export_inflight = false;
    return ASPH_OK;
}

// Device staging of one export: positions, velocities (pending half-kick applied), densities, radii, ids.
struct ExportStage {
    float4* pos;
    float4* vel;
    float* rho;
    float* rad;
    uint32_t* ids;
    size_t n;
};

// Writes the requested export arrays of the current particles into the staging buffer (kept across calls, grown on
// demand, so that a per-frame export allocates nothing), on the simulation's stream.
asph_status export_stage(asph_simulation* s, const void* positions, const void* velocities, const void* densities,
                         const void* radii, const void* ids, ExportStage& x) {
    const size_t n = s->n;
    const size_t bytes = n * (16 + 16 + 4 + 4 + 4);
    if (bytes > s->stage_bytes) {
        asph_status st = export_settle(s);
        if (st != ASPH_OK) return st;
        CK(cudaStreamSynchronize(s->stream));
        dfree(s->stage);
        s->stage = nullptr;
        s->stage_bytes = 0;
        if ((st = dalloc(s->stage, bytes)) != ASPH_OK) return st;
        s->stage_bytes = bytes;
    }
    x.n = n;
    x.pos = reinterpret_cast<float4*>(s->stage);
    x.vel = x.pos + n;
    x.rho = reinterpret_cast<float*>(x.vel + n);
    x.rad = x.rho + n;
    x.ids = reinterpret_cast<uint32_t*>(x.rad + n);
    k_export<<<blocks_for((uint32_t)n), 256, 0, s->stream>>>(s->args(s->cur), s->pending_half, s->has_pending ? 1 : 0,
                                                            positions ? x.pos : nullptr, velocities ? x.vel : nullptr,
                                                            densities ? x.rho : nullptr, radii ? x.rad : nullptr,
                                                            ids ? x.ids : nullptr);
    CK_LAUNCH("k_export");
    s->launches++;
    return ASPH_OK;
}

// Device-to-host copies of a staged export on `stream`.
asph_status export_copies(cudaStream_t stream, const ExportStage& x, float* positions, float* velocities,
                          float* densities, float* radii, uint32_t* ids) {
    if (positions) CK(cudaMemcpyAsync(positions, x.pos, 16 * x.n, cudaMemcpyDeviceToHost, stream));
    if (velocities) CK(cudaMemcpyAsync(velocities, x.vel, 16 * x.n, cudaMemcpyDeviceToHost, stream));
    if (densities) CK(cudaMemcpyAsync(densities, x.rho, 4 * x.n, cudaMemcpyDeviceToHost, stream));
    if (radii) CK(cudaMemcpyAsync(radii, x.rad, 4 * x.n, cudaMemcpyDeviceToHost, stream));
    if (ids) CK(cudaMemcpyAsync(ids, x.ids, 4 * x.n, cudaMemcpyDeviceToHost, stream));
    return ASPH_OK;
}

void destroy(asph_simulation* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->own_graph) scene_graph_free(s->own_graph);
    s->own_graph = nullptr;
    dfree(s->arena);  // the fixed-size buffers (carve_fixed)
    dfree(s->nbr_ent);
    dfree(s->cell_block);  // the five sub-cell tables
    dfree(s->hmax_ref);
    dfree(s->bpos);
    dfree(s->bfric);
    dfree(s->brefflag);
    dfree(s->dbg_ids);
    dfree(s->stage);
    if (s->h_ctr) cudaFreeHost(s->h_ctr);  // h_small lies in the same allocation
    for (auto& e : s->events) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    for (auto e : s->event_pool) cudaEventDestroy(e);
    if (s->aux) cudaStreamSynchronize(s->aux);
    if (s->copy) cudaStreamSynchronize(s->copy);
    if (s->ev_export_ready) cudaEventDestroy(s->ev_export_ready);
    if (s->ev_export_done) cudaEventDestroy(s->ev_export_done);
    if (s->copy) cudaStreamDestroy(s->copy);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_main) cudaEventDestroy(s->ev_main);
    if (s->ev_aux) cudaEventDestroy(s->ev_aux);
    if (s->ev_refine) cudaEventDestroy(s->ev_refine);
    if (s->aux) cudaStreamDestroy(s->aux);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    delete s;
    (void)cudaGetLastError();
}

}  // namespace

// ================================================================================================ C ABI
extern "C" {

uint32_t asph_abi_version(void) { return ASPH_ABI_VERSION; }

const char* asph_status_string(asph_status s) {
    switch (s) {
        case ASPH_OK: return "ok";
        case ASPH_ERR_INVALID_ARGUMENT: return "invalid argument";
        case ASPH_ERR_CUDA: return "CUDA error";
        case ASPH_ERR_OUT_OF_MEMORY: return "out of device memory";
        case ASPH_ERR_CAPACITY: return "capacity exceeded";
        case ASPH_ERR_DEVICE_CHECK: return "device check failed";
        case ASPH_ERR_UNSUPPORTED: return "unsupported";
        case ASPH_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

const char* asph_last_error(void) { return g_last_error.c_str(); }

void asph_refinement_parameters_default(asph_refinement_parameters* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->enabled = 0;
    p->min_mass_ratio = 0.3f;
    p->max_mass_ratio = 8.0f;
    p->max_particle_count = 1000000;
    p->max_batch_ratio = 0.2f;
    p->initial_cooldown = 10;
    p->cooldown = 10;
    p->criterion = ASPH_CRITERION_VELOCITY;
    p->split_epsilon = 0.65f;
    p->split_alpha = 0.70f;
    p->split_center_mass_ratio = 0.077f;
    p->split_vertex_mass_ratio = 0.077f;
    p->velocity_split_min_speed = 2.0f;
    p->velocity_merge_max_speed = 0.1f;
    p->vorticity_split_min = 1.0f;
    p->vorticity_merge_max = 0.3f;
    p->curvature_split_min = 2.0f;
    p->curvature_merge_max = 0.6f;
    p->interface_split_distance_ratio = 0.05f;
    p->interface_merge_distance_ratio = 0.15f;
    p->free_surface_split_deficit = 0.25f;
    p->free_surface_merge_deficit = 0.05f;
}

// ---------------------------------------------------------------------------------------------- memory
asph_status asph_import_buffer_fd(int fd, size_t size, asph_memory** out) {
    API_ENTRY();
    if (!out || fd < 0 || size == 0) return fail(ASPH_ERR_INVALID_ARGUMENT, "import needs an fd, a size and out");
    *out = nullptr;
    cudaExternalMemoryHandleDesc hd;
    std::memset(&hd, 0, sizeof(hd));
    hd.type = cudaExternalMemoryHandleTypeOpaqueFd;
    hd.handle.fd = fd;
    hd.size = size;
    cudaExternalMemory_t ext = nullptr;
    CK(cudaImportExternalMemory(&ext, &hd));
    cudaExternalMemoryBufferDesc bd;
    std::memset(&bd, 0, sizeof(bd));
    bd.offset = 0;
    bd.size = size;
    void* ptr = nullptr;
    cudaError_t e = cudaExternalMemoryGetMappedBuffer(&ptr, ext, &bd);
    if (e != cudaSuccess) {
        cudaDestroyExternalMemory(ext);
        return cuda_fail(e, "cudaExternalMemoryGetMappedBuffer");
    }
    asph_memory* m = new (std::nothrow) asph_memory;
    if (!m) {
        cudaFree(ptr);
        cudaDestroyExternalMemory(ext);
        return fail(ASPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    m->ptr = ptr;
    m->size = size;
    m->ext = ext;
    *out = m;
    return ASPH_OK;
}

asph_status asph_memory_allocate(size_t size, asph_memory** out) {
    API_ENTRY();
    if (!out || size == 0) return fail(ASPH_ERR_INVALID_ARGUMENT, "allocation needs a size and out");
    *out = nullptr;
    void* p = nullptr;
    CK(cudaMalloc(&p, size));
    CK(cudaMemset(p, 0, size));
    asph_memory* m = new (std::nothrow) asph_memory;
    if (!m) {
        cudaFree(p);
        return fail(ASPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    m->ptr = p;
    m->size = size;
    *out = m;
    return ASPH_OK;
}

asph_status asph_memory_device_pointer(const asph_memory* mem, void** out) {
    API_ENTRY();
    if (!mem || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = mem->ptr;
    return ASPH_OK;
}

asph_status asph_memory_size(const asph_memory* mem, size_t* out) {
    API_ENTRY();
    if (!mem || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = mem->size;
    return ASPH_OK;
}

void asph_memory_release(asph_memory* mem) {
    if (!mem) return;
    if (mem->ptr) cudaFree(mem->ptr);
    if (mem->ext) cudaDestroyExternalMemory(mem->ext);
    delete mem;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------- simulation
// createSimulation; the boundary comes from host particles or, when `walls` is given, from walls generated on the
// device (their count is walls->n; boundary / boundary_count are then unused).
// With the CUDA runtime's lazy loading (the default), a kernel is loaded at its first launch, which then waits for
// the load; the refinement and read-out kernels first run many frames into a simulation, inside its step loop.
// They are loaded once per process when the first simulation is created instead.
static void preload_kernels() {
    static std::once_flag once;
    std::call_once(once, [] {
        const void* kernels[] = {
            (const void*)k_merge_score,    (const void*)k_split_score,      (const void*)k_select_ids,
            (const void*)k_select_scores,  (const void*)k_merge_limits,     (const void*)k_cand_init,
            (const void*)k_mark_eligible,  (const void*)k_merge_candidates, (const void*)k_merge_candidates_heavy,
            (const void*)k_merge_pairs,    (const void*)k_compact_count,    (const void*)k_compact_scan,
            (const void*)k_compact_scatter, (const void*)k_split_limits,    (const void*)k_split_apply,
            (const void*)k_refine_finish,  (const void*)k_cells_only,       (const void*)k_export,
            (const void*)k_select_split_ids,
            (const void*)k_totals,         (const void*)k_density_info,     (const void*)k_reduce_rows,
            (const void*)k_neighbor_counts};
        for (const void* k : kernels) {
            cudaFuncAttributes attr;
            (void)cudaFuncGetAttributes(&attr, k);
        }
        (void)cudaGetLastError();
    });
}

// The fixed-size device buffers of a simulation are carved from one allocation: creation made ~35 cudaMalloc calls
// otherwise, 50-100 us each whatever the size. Each buffer starts on a 256-byte boundary; a first pass with no base
// measures the total. (The neighbour rows, cell tables and boundary arrays, which are reallocated, stay apart.)
struct Carver {
    uint8_t* base = nullptr;
    size_t used = 0;
    template <class T>
    void take(T*& p, size_t count) {
        used = (used + 255) & ~size_t(255);
        p = base ? reinterpret_cast<T*>(base + used) : nullptr;
        used += sizeof(T) * std::max<size_t>(count, 1);
    }
};

static void carve_fixed(asph_simulation* s, Carver& c, uint32_t sort_items) {
    const size_t C = s->cap;
    for (int k = 0; k < 2; k++) {
        c.take(s->set[k].ph, C);
        c.take(s->set[k].vm, C);
        c.take(s->set[k].acc, C);
        c.take(s->set[k].rp, C);
        c.take(s->set[k].rad, C);
        c.take(s->set[k].id, C);
    }
    c.take(s->kc, C);
    c.take(s->pq, C);
    c.take(s->fr, C);
    c.take(s->nbr_cnt, C);
    c.take(s->nbr_bcnt, C);
    c.take(s->heavy_idx, C);
    c.take(s->heavy_n, 1);
    c.take(s->fheavy_idx, C);
    c.take(s->fheavy_n, 4);
    c.take(s->dover_idx, C);
    c.take(s->drow_idx, C);
    c.take(s->frow_idx, C);
    c.take(s->pool, (size_t)s->pool_slots * 32 * kPoolLaneEntries);
    c.take(s->pool_cnt, (size_t)s->pool_slots * 32);
    c.take(s->keys, sort_items);
    c.take(s->vals, sort_items);
    uint8_t* mem = nullptr;
    c.take(mem, sort_scratch_bytes(sort_items));
    s->sort_mem = mem;
    c.take(s->ex, 4);
    c.take(s->q3, 2);
    c.take(s->err, 1);
    c.take(s->d_count, 2);
    c.take(s->red, kRedBytes);
    if (s->adaptive) {
        c.take(s->score, C);
        c.take(s->cand, C);
        c.take(s->flag, C);
        c.take(s->ctr, kCtrNum);
        c.take(s->slot0, 1);
        c.take(s->block_counts, blocks_for((uint32_t)C));
        c.take(s->rkeys, 2 * C);
    }
}

static asph_status create_impl(const asph_parameters* parameters, const float* positions, uint32_t count,
                               const asph_fluid_buffers* fluid_buffers, const asph_boundary_buffers* boundary_buffers,
                               const asph_boundary_particle* boundary, uint32_t boundary_count,
                               const DeviceWalls* walls, const asph_refinement_parameters* refinement,
                               uint32_t max_fluid_capacity, uint32_t max_boundary_capacity, asph_simulation** out) {
    if (walls) {
        boundary = nullptr;
        boundary_count = walls->n;
    }
    if (!parameters || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "parameters and out are required");
    *out = nullptr;
    if (count > 0 && !positions) return fail(ASPH_ERR_INVALID_ARGUMENT, "positions are required");
    preload_kernels();
    if (boundary_count > 0 && !boundary && !walls)
        return fail(ASPH_ERR_INVALID_ARGUMENT, "boundary particles are required");
    const asph_parameters& P = *parameters;
    if (!(P.base_smoothing_radius > 0.0f) || !(P.rest_density > 0.0f) || !(P.speed_of_sound > 0.0f) ||
        !(P.base_particle_mass > 0.0f))
        return fail(ASPH_ERR_INVALID_ARGUMENT, "smoothing radius, rest density, speed of sound and mass must be > 0");
    if (P.viscosity_model > 1u || P.boundary_mode > 1u)
        return fail(ASPH_ERR_INVALID_ARGUMENT, "unknown viscosity model or boundary mode");
    const bool adaptive = refinement && refinement->enabled;
    if (adaptive) {
        if (refinement->cooldown == 0) return fail(ASPH_ERR_INVALID_ARGUMENT, "refinement cooldown must be > 0");
        if (refinement->criterion > 3u) return fail(ASPH_ERR_INVALID_ARGUMENT, "unknown refinement criterion");
        if (refinement->criterion == ASPH_CRITERION_FREE_SURFACE &&
            !(refinement->free_surface_merge_deficit > 0.0f && refinement->free_surface_split_deficit > 0.0f))
            return fail(ASPH_ERR_INVALID_ARGUMENT, "free-surface deficits must be positive");
        if (P.boundary_mode == ASPH_BOUNDARY_PERIODIC)
            return fail(ASPH_ERR_UNSUPPORTED, "refinement in a periodic box is not supported");
    }
    // AdaptiveSphSimulation sizes the fluid arrays by maxParticleCount (AdaptiveSphSimulation.cu:37)
    const uint32_t cap = adaptive ? refinement->max_particle_count : std::max(max_fluid_capacity, count);
    if (count > cap) return fail(ASPH_ERR_CAPACITY, "more particles than the fluid capacity");
    if (cap > (1u << 30)) return fail(ASPH_ERR_UNSUPPORTED, "fluid capacity above 2^30");
    if (P.boundary_mode == ASPH_BOUNDARY_PERIODIC && cap >= (1u << 27))
        return fail(ASPH_ERR_UNSUPPORTED, "a periodic box holds at most 2^27 - 1 particles");
    asph_simulation* s = new (std::nothrow) asph_simulation;
    static std::atomic<uint64_t> next_serial{1};
    if (s) s->serial = next_serial.fetch_add(1);
    if (!s) return fail(ASPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->P = P;
    if (adaptive) s->R = *refinement;
    s->adaptive = adaptive;
    s->tpb = P.threads_per_block ? P.threads_per_block : 256u;
    s->cap = std::max(cap, 1u);
    s->n = count;
    s->next_id = count;
    asph_status st = make_grid(P, s->grid);
    if (st != ASPH_OK) {
        delete s;
        return st;
    }
    make_phys(P, s->phys);
    if (fluid_buffers) {
        s->fbuf = *fluid_buffers;
        s->have_fbuf = true;
    }
    if (boundary_buffers) {
        s->bbuf = *boundary_buffers;
        s->have_bbuf = true;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        destroy(s);
        return cuda_fail(e, "cudaStreamCreate");
    }
    s->stream = s->own_stream;
    // the heavy-particle kernels run few, long warps: their stream gets the highest priority so that their blocks
    // are dispatched ahead of the ordinary kernels' and their latency overlaps the ordinary work
    int prio_least = 0, prio_greatest = 0;
    e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->aux, cudaStreamNonBlocking, prio_greatest);
    s->heavy_priority = prio_greatest;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_main, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_aux, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_refine, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        destroy(s);
        return cuda_fail(e, "aux stream");
    }
#define TRY(x)                     \
    if ((st = (x)) != ASPH_OK) {   \
        destroy(s);                \
        return st;                 \
    }
    const uint32_t C = s->cap;
    const uint32_t sort_items = std::max(C, std::max(boundary_count, max_boundary_capacity));
    s->pool_slots = std::min<uint32_t>(kPoolSlots, std::max<uint32_t>(64u, C / 128u));
    {
        Carver plan;
        carve_fixed(s, plan, sort_items);
        TRY(dalloc(s->arena, plan.used));
        Carver take{s->arena};
        carve_fixed(s, take, sort_items);
        sort_scratch_bind(s->ss, s->sort_mem, sort_items);
    }
    s->device_bytes = device_bytes_for(C, sort_items, s->grid.ncells,
                                       (uint32_t)(s->grid.gs[0] * s->grid.gs[1] * s->grid.gs[2]), boundary_count,
                                       adaptive);
    s->rows_cap = rows_for(count, C);
    TRY(dalloc(s->nbr_ent, (size_t)kListEntries * s->rows_cap));
    TRY(alloc_cells(s));
    // the pinned read-back words: 64 counters, then 16 64-bit values, in one allocation
    e = cudaMallocHost(reinterpret_cast<void**>(&s->h_ctr), sizeof(uint32_t) * 64 + sizeof(uint64_t) * 16);
    if (e != cudaSuccess) {
        destroy(s);
        return cuda_fail(e, "cudaMallocHost");
    }
    s->h_small = reinterpret_cast<decltype(s->h_small)>(s->h_ctr + 64);
    CK(cudaMemsetAsync(s->err, 0, sizeof(uint32_t), s->stream));
    s->bcap = 0;
    TRY(walls ? setup_boundary_device(s, walls->pos, walls->psi, walls->n)
              : setup_boundary(s, boundary, boundary_count, true));
    if (walls) s->launches += walls->launches;
    if (count > 0) {
        // the caller's positions, read in place where the device reads host memory coherently, else copied first
        float4* d_pos = nullptr;
        const float4* src = reinterpret_cast<const float4*>(positions);
        if (!device_reads_host_in_place(positions, alignof(float4))) {
            TRY(dalloc(d_pos, count));
            e = cudaMemcpyAsync(d_pos, positions, sizeof(float4) * count, cudaMemcpyHostToDevice, s->stream);
            src = d_pos;
        }
        if (e == cudaSuccess) {
            k_init_state<<<blocks_for(count), 256, 0, s->stream>>>(s->args(s->cur), src, P.base_particle_radius,
                                                                   P.base_smoothing_radius, P.base_particle_mass);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        dfree(d_pos);
        if (e != cudaSuccess) {
            destroy(s);
            return cuda_fail(e, "initial upload");
        }
        s->launches++;
    }
    TRY(upload_count(s));
    e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        destroy(s);
        return cuda_fail(e, "create");
    }
#undef TRY
    *out = s;
    return ASPH_OK;
}

namespace {
asph_status graph_step(asph_simulation* s, SceneGraph& g, float dt, AdvanceStats& stats);
}  // namespace

// A plain step (no refinement pass due, a pending half-kick to fuse, particles present) of a simulation of up to
// kGraphStepParticles particles replays a captured graph, which saves the launch gaps of ~20 dependent kernels (at
// 128k particles a step takes 0.32 ms from a graph against 0.36 ms launched one by one). Larger simulations launch
// eagerly: their device time hides the gaps (1.67 against 1.69 ms per step at 1M), and the two captures (one per
// buffer parity, ~1 ms each) would cost more than they save over the first hundreds of steps. Not while per-stage
// timing is on (its events belong to eager launches), not on the legacy or per-thread default stream (they cannot
// be captured), and not while the caller captures the stream.
constexpr uint32_t kGraphStepParticles = 262144;
static bool plain_step_graphable(asph_simulation* s) {
    if (s->n == 0 || s->n > kGraphStepParticles || !s->has_pending || s->timing || refinement_due(s)) return false;
    if (s->stream == nullptr || s->stream == cudaStreamLegacy || s->stream == cudaStreamPerThread) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return false;
    return true;
}

extern "C" {

asph_status asph_simulation_create(const asph_parameters* parameters, const float* positions, uint32_t count,
                                   const asph_fluid_buffers* fluid_buffers,
                                   const asph_boundary_buffers* boundary_buffers,
                                   const asph_boundary_particle* boundary, uint32_t boundary_count,
                                   const asph_refinement_parameters* refinement, uint32_t max_fluid_capacity,
                                   uint32_t max_boundary_capacity, asph_simulation** out) {
    API_ENTRY();
    return create_impl(parameters, positions, count, fluid_buffers, boundary_buffers, boundary, boundary_count,
                       nullptr, refinement, max_fluid_capacity, max_boundary_capacity, out);
}

asph_status asph_simulation_create_with_walls(const asph_parameters* parameters, const float* positions,
                                              uint32_t count, const asph_fluid_buffers* fluid_buffers,
                                              const asph_boundary_buffers* boundary_buffers, float wall_spacing,
                                              const asph_refinement_parameters* refinement,
                                              uint32_t max_fluid_capacity, uint32_t max_boundary_capacity,
                                              asph_simulation** out) {
    API_ENTRY();
    if (!parameters || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "parameters and out are required");
    *out = nullptr;
    DeviceWalls w;
    asph_status st = generate_walls_device(parameters->domain, wall_spacing, parameters->rest_density,
                                           parameters->base_smoothing_radius, nullptr, w);
    if (st != ASPH_OK) return st;
    st = create_impl(parameters, positions, count, fluid_buffers, boundary_buffers, nullptr, 0, &w, refinement,
                     max_fluid_capacity, std::max(max_boundary_capacity, w.n), out);
    free_walls(w);
    return st;
}

void asph_simulation_destroy(asph_simulation* sim) { destroy(sim); }

asph_status asph_simulation_step_async(asph_simulation* sim, float delta_time) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    if (plain_step_graphable(sim)) {
        if (!sim->own_graph && !(sim->own_graph = scene_graph_new()))
            return fail(ASPH_ERR_OUT_OF_MEMORY, "step graph");
        if (!std::isfinite(delta_time)) return fail(ASPH_ERR_INVALID_ARGUMENT, "delta time must be finite");
        AdvanceStats stats;
        return graph_step(sim, *sim->own_graph, delta_time, stats);
    }
    return run_step(sim, delta_time, ASPH_STAGE_ALL);
}

asph_status asph_simulation_update(asph_simulation* sim, float delta_time) {
    API_ENTRY();
    asph_status st = asph_simulation_step_async(sim, delta_time);
    if (st != ASPH_OK) return st;
    return check_errors(sim, true);
}

asph_status asph_simulation_run_stages(asph_simulation* sim, float delta_time, uint32_t last_stage) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    if (last_stage < ASPH_STAGE_INTEGRATE || last_stage > ASPH_STAGE_ALL)
        return fail(ASPH_ERR_INVALID_ARGUMENT, "unknown stage");
    asph_status st = run_step(sim, delta_time, last_stage);
    if (st != ASPH_OK) return st;
    return check_errors(sim, true);
}

asph_status asph_simulation_synchronize(asph_simulation* sim) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    asph_status st = export_settle(sim);
    if (st != ASPH_OK) return st;
    return check_errors(sim, true);
}

// Fixed-order FP64 reduction of the current state into h[0..ncols): k_totals or k_density_info, then k_reduce_rows.
static asph_status reduce_state(asph_simulation* sim, bool density_info, float threshold, double* h) {
    double* out = reinterpret_cast<double*>(sim->red);
    double* rows = out + 8;
    const uint32_t blocks = std::min<uint32_t>(kRedBlocks, blocks_for(sim->n));
    uint32_t ncols, min_mask, max_mask;
    if (density_info) {
        k_density_info<<<blocks, 256, 0, sim->stream>>>(sim->args(sim->cur), threshold, sim->P.rest_density, rows);
        CK_LAUNCH("k_density_info");
        ncols = 6, min_mask = 1u << 1, max_mask = 1u << 2;
    } else {
        k_totals<<<blocks, 256, 0, sim->stream>>>(sim->args(sim->cur), sim->pending_half, sim->has_pending ? 1 : 0,
                                                  rows);
        CK_LAUNCH("k_totals");
        ncols = 7, min_mask = 1u << 6, max_mask = 0;
    }
    k_reduce_rows<<<1, 256, 0, sim->stream>>>(rows, blocks, ncols, min_mask, max_mask, out);
    CK_LAUNCH("k_reduce_rows");
    sim->launches += 2;
    CK(cudaMemcpyAsync(h, out, sizeof(double) * ncols, cudaMemcpyDeviceToHost, sim->stream));
    CK(cudaStreamSynchronize(sim->stream));
    return ASPH_OK;
}

asph_status asph_simulation_totals(asph_simulation* sim, asph_totals* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(out, 0, sizeof(*out));
    out->count = sim->n;
    if (sim->n == 0) return ASPH_OK;
    double h[8];
    asph_status st = reduce_state(sim, false, 0.0f, h);
    if (st != ASPH_OK) return st;
    out->mass = h[0];
    out->momentum[0] = h[1];
    out->momentum[1] = h[2];
    out->momentum[2] = h[3];
    out->kinetic_energy = h[4];
    out->volume = h[5];
    return ASPH_OK;
}

asph_status asph_simulation_step_cfl(asph_simulation* sim, float cfl, float dt_max, float* dt_used) {
    API_ENTRY();
    if (!sim || !(cfl > 0.0f)) return fail(ASPH_ERR_INVALID_ARGUMENT, "simulation and cfl > 0 required");
    float dt = dt_max > 0.0f ? dt_max : 3.402823466e38f;
    if (sim->n > 0) {
        double h[8];
        asph_status st = reduce_state(sim, false, 0.0f, h);
        if (st != ASPH_OK) return st;
        const float m = (float)h[6];  // a float converted to double and back: exact
        const float c = cfl * m;
        if (c < dt) dt = c;
    }
    if (!(dt < 3.0e38f)) return fail(ASPH_ERR_INVALID_ARGUMENT, "no particles and no dt_max");
    if (dt_used) *dt_used = dt;
    if (!std::isfinite(dt)) return fail(ASPH_ERR_INVALID_ARGUMENT, "delta time must be finite");
    return run_step(sim, dt, ASPH_STAGE_ALL);  // eager: dt changes every step, a graph would be captured each time
}

asph_status asph_simulation_update_domain(asph_simulation* sim, const asph_domain* domain,
                                          const asph_boundary_particle* boundary, uint32_t boundary_count) {
    API_ENTRY();
    if (!sim || !domain) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    if (boundary_count > 0 && !boundary) return fail(ASPH_ERR_INVALID_ARGUMENT, "boundary particles are required");
    CK(cudaStreamSynchronize(sim->stream));
    asph_parameters P = sim->P;
    P.domain = *domain;
    GridDev g;
    asph_status st = make_grid(P, g);
    if (st != ASPH_OK) return st;
    if (boundary_count > sim->ss.max_items)
        return fail(ASPH_ERR_CAPACITY, "more boundary particles than the sort capacity of this simulation");
    sim->P = P;
    sim->grid = g;
    sim->generation++;
    if ((st = alloc_cells(sim)) != ASPH_OK) return st;
    if ((st = setup_boundary(sim, boundary, boundary_count)) != ASPH_OK) return st;
    sim->grid_valid = false;
    return check_errors(sim, true);
}

asph_status asph_simulation_fluid_count(const asph_simulation* sim, uint32_t* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = sim->n;
    return ASPH_OK;
}

asph_status asph_simulation_boundary_count(const asph_simulation* sim, uint32_t* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = sim->nb;
    return ASPH_OK;
}

asph_status asph_simulation_neighbor_counts(asph_simulation* sim, uint32_t* counts, uint32_t capacity) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    if (counts && capacity < sim->n) return fail(ASPH_ERR_CAPACITY, "counts array too small");
    if (sim->n == 0) return ASPH_OK;
    asph_status st;
    if ((st = ensure_grid(sim)) != ASPH_OK) return st;
    uint32_t* d = nullptr;
    unsigned long long* tot = nullptr;
    if ((st = dalloc(d, sim->n)) != ASPH_OK) return st;
    if ((st = dalloc(tot, 1)) != ASPH_OK) {
        dfree(d);
        return st;
    }
    CK(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), sim->stream));
    k_neighbor_counts<<<blocks_for(sim->n), 256, 0, sim->stream>>>(sim->args(sim->cur), sim->cells(), d, tot);
    CK_LAUNCH("k_neighbor_counts");
    sim->launches++;
    if (counts) CK(cudaMemcpyAsync(counts, d, sizeof(uint32_t) * sim->n, cudaMemcpyDeviceToHost, sim->stream));
    CK(cudaStreamSynchronize(sim->stream));
    dfree(d);
    dfree(tot);
    return ASPH_OK;
}

asph_status asph_simulation_average_neighbor_count(asph_simulation* sim, float* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = 0.0f;
    if (sim->n == 0) return ASPH_OK;
    asph_status st;
    if ((st = ensure_grid(sim)) != ASPH_OK) return st;
    unsigned long long* tot = nullptr;
    if ((st = dalloc(tot, 1)) != ASPH_OK) return st;
    CK(cudaMemsetAsync(tot, 0, sizeof(unsigned long long), sim->stream));
    k_neighbor_counts<<<blocks_for(sim->n), 256, 0, sim->stream>>>(sim->args(sim->cur), sim->cells(), nullptr, tot);
    CK_LAUNCH("k_neighbor_counts");
    sim->launches++;
    unsigned long long h = 0;
    CK(cudaMemcpyAsync(&h, tot, sizeof(h), cudaMemcpyDeviceToHost, sim->stream));
    CK(cudaStreamSynchronize(sim->stream));
    dfree(tot);
    // the reference accumulates a uint32 total (SphSimulation.cu:237-247)
    *out = (float)(uint32_t)h / (float)sim->n;
    return ASPH_OK;
}

asph_status asph_simulation_density_info(asph_simulation* sim, float threshold, asph_density_info* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    std::memset(out, 0, sizeof(*out));
    out->rest_density = sim->P.rest_density;
    out->min_density = 3.402823466e38f;
    out->max_density = -3.402823466e38f;
    if (sim->n == 0) {
        out->average_density = NAN;  // 0 / 0 as in the reference (SphSimulation.cu:283)
        return ASPH_OK;
    }
    double h[8];
    asph_status st = reduce_state(sim, true, threshold, h);
    if (st != ASPH_OK) return st;
    out->min_density = (float)h[1];
    out->max_density = (float)h[2];
    out->average_density = (float)(h[0] / (double)sim->n);
    const uint32_t hc[3] = {(uint32_t)h[3], (uint32_t)h[4], (uint32_t)h[5]};
    out->under_density_count = hc[0];
    out->normal_density_count = hc[1];
    out->over_density_count = hc[2];
    return ASPH_OK;
}

asph_status asph_simulation_enable_adaptive_refinement(asph_simulation* sim) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    if (sim->adaptive) sim->frame = sim->R.initial_cooldown;
    return ASPH_OK;
}

asph_status asph_simulation_export(asph_simulation* sim) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    if (!sim->have_fbuf) return ASPH_OK;
    const asph_fluid_buffers& f = sim->fbuf;
    const size_t n = sim->n;
    auto ptr_if = [&](const asph_memory* m, size_t bytes) -> void* {
        return (m && m->ptr && m->size >= bytes) ? m->ptr : nullptr;
    };
    if (n > 0) {
        k_export<<<blocks_for(sim->n), 256, 0, sim->stream>>>(
            sim->args(sim->cur), sim->pending_half, sim->has_pending ? 1 : 0,
            static_cast<float4*>(ptr_if(f.positions, 16 * n)), static_cast<float4*>(ptr_if(f.velocities, 16 * n)),
            static_cast<float*>(ptr_if(f.densities, 4 * n)), static_cast<float*>(ptr_if(f.radii, 4 * n)), nullptr);
        CK_LAUNCH("k_export");
        sim->launches++;
    }
    return check_errors(sim, true);
}

asph_status asph_simulation_export_host(asph_simulation* sim, float* positions, float* velocities, float* densities,
                                        float* radii, uint32_t* ids, uint32_t capacity) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    const uint32_t n = sim->n;
    if (capacity < n) return fail(ASPH_ERR_CAPACITY, "host arrays too small");
    asph_status st = export_settle(sim);
    if (st != ASPH_OK) return st;
    if (n == 0) return ASPH_OK;
    ExportStage x;
    if ((st = export_stage(sim, positions, velocities, densities, radii, ids, x)) != ASPH_OK) return st;
    if ((st = export_copies(sim->stream, x, positions, velocities, densities, radii, ids)) != ASPH_OK) return st;
    CK(cudaStreamSynchronize(sim->stream));
    return check_errors(sim, false);
}

asph_status asph_simulation_export_host_async(asph_simulation* sim, float* positions, float* velocities,
                                              float* densities, float* radii, uint32_t* ids, uint32_t capacity) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    const uint32_t n = sim->n;
    if (capacity < n) return fail(ASPH_ERR_CAPACITY, "host arrays too small");
    if (!sim->copy) {
        cudaError_t e = cudaStreamCreateWithFlags(&sim->copy, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sim->ev_export_ready, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sim->ev_export_done, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(e, "export stream");
    }
    if (n == 0) return ASPH_OK;
    // the staging buffer is reused: the export kernel waits (on the device) for the previous copies
    if (sim->export_inflight) CK(cudaStreamWaitEvent(sim->stream, sim->ev_export_done, 0));
    ExportStage x;
    asph_status st = export_stage(sim, positions, velocities, densities, radii, ids, x);
    if (st != ASPH_OK) return st;
    CK(cudaEventRecord(sim->ev_export_ready, sim->stream));
    CK(cudaStreamWaitEvent(sim->copy, sim->ev_export_ready, 0));
    if ((st = export_copies(sim->copy, x, positions, velocities, densities, radii, ids)) != ASPH_OK) return st;
    CK(cudaEventRecord(sim->ev_export_done, sim->copy));
    sim->export_inflight = true;
    return ASPH_OK;
}

asph_status asph_simulation_export_wait(asph_simulation* sim) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    asph_status st = export_settle(sim);
    if (st != ASPH_OK) return st;
    return check_errors(sim, false);
}

asph_status asph_simulation_device_errors(asph_simulation* sim, uint32_t* out, int clear) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    CK(cudaStreamSynchronize(sim->stream));
    CK(cudaMemcpy(sim->h_ctr, sim->err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    *out = sim->h_ctr[0];
    if (clear) CK(cudaMemset(sim->err, 0, sizeof(uint32_t)));
    return ASPH_OK;
}

asph_status asph_simulation_set_stream(asph_simulation* sim, void* cuda_stream) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    CK(cudaStreamSynchronize(sim->stream));
    sim->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : sim->own_stream;
    return ASPH_OK;
}

asph_status asph_simulation_state_info(asph_simulation* sim, asph_state_info* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    out->count = sim->n;
    out->capacity = sim->cap;
    out->frame = sim->frame;
    out->next_id = sim->next_id;
    out->pending_half_dt = sim->pending_half;
    out->has_pending = sim->has_pending ? 1u : 0u;
    return ASPH_OK;
}

asph_status asph_simulation_read_fluid(asph_simulation* sim, float* positions, float* velocities,
                                       float* accelerations, float* densities, float* radii, float* smoothing_radii,
                                       float* masses, uint32_t* ids, uint32_t capacity) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    const uint32_t n = sim->n;
    if (capacity < n) return fail(ASPH_ERR_CAPACITY, "host arrays too small");
    if (n == 0) return ASPH_OK;
    uint8_t* stage = nullptr;
    const size_t bytes = (size_t)n * (16 * 3 + 4 * 5);
    asph_status st;
    if ((st = dalloc(stage, bytes)) != ASPH_OK) return st;
    float4* p = reinterpret_cast<float4*>(stage);
    float4* v = p + n;
    float4* a = v + n;
    float* rho = reinterpret_cast<float*>(a + n);
    float* rad = rho + n;
    float* h = rad + n;
    float* m = h + n;
    uint32_t* id = reinterpret_cast<uint32_t*>(m + n);
    k_read_state<<<blocks_for(n), 256, 0, sim->stream>>>(sim->args(sim->cur), p, v, a, rho, rad, h, m, id);
    CK_LAUNCH("k_read_state");
    sim->launches++;
    struct Item {
        void* dst;
        const void* src;
        size_t b;
    } items[] = {{positions, p, 16}, {velocities, v, 16}, {accelerations, a, 16}, {densities, rho, 4},
                 {radii, rad, 4},    {smoothing_radii, h, 4}, {masses, m, 4},    {ids, id, 4}};
    for (auto& it : items)
        if (it.dst) CK(cudaMemcpyAsync(it.dst, it.src, it.b * n, cudaMemcpyDeviceToHost, sim->stream));
    CK(cudaStreamSynchronize(sim->stream));
    dfree(stage);
    return ASPH_OK;
}

asph_status asph_simulation_write_fluid(asph_simulation* sim, const asph_state_info* info, const float* positions,
                                        const float* velocities, const float* accelerations, const float* densities,
                                        const float* radii, const float* smoothing_radii, const float* masses,
                                        const uint32_t* ids) {
    API_ENTRY();
    if (!sim || !info) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    const uint32_t n = info->count;
    if (n > sim->cap) return fail(ASPH_ERR_CAPACITY, "more particles than the fluid capacity");
    if (n > 0 && (!positions || !velocities || !accelerations || !densities || !radii || !smoothing_radii ||
                  !masses || !ids))
        return fail(ASPH_ERR_INVALID_ARGUMENT, "all state arrays are required");
    CK(cudaStreamSynchronize(sim->stream));
    sim->n = n;
    sim->generation++;
    if (n > 0) {
        uint8_t* stage = nullptr;
        const size_t bytes = (size_t)n * (16 * 3 + 4 * 5);
        asph_status st;
        if ((st = dalloc(stage, bytes)) != ASPH_OK) return st;
        float4* p = reinterpret_cast<float4*>(stage);
        float4* v = p + n;
        float4* a = v + n;
        float* rho = reinterpret_cast<float*>(a + n);
        float* rad = rho + n;
        float* h = rad + n;
        float* m = h + n;
        uint32_t* id = reinterpret_cast<uint32_t*>(m + n);
        struct Item {
            void* dst;
            const void* src;
            size_t b;
        } items[] = {{p, positions, 16}, {v, velocities, 16}, {a, accelerations, 16}, {rho, densities, 4},
                     {rad, radii, 4},    {h, smoothing_radii, 4}, {m, masses, 4},     {id, ids, 4}};
        for (auto& it : items) CK(cudaMemcpyAsync(it.dst, it.src, it.b * n, cudaMemcpyHostToDevice, sim->stream));
        k_write_state<<<blocks_for(n), 256, 0, sim->stream>>>(sim->args(sim->cur), p, v, a, rho, rad, h, m, id);
        CK_LAUNCH("k_write_state");
        sim->launches++;
        CK(cudaStreamSynchronize(sim->stream));
        dfree(stage);
    }
    sim->frame = info->frame;
    sim->next_id = info->next_id;
    sim->pending_half = info->pending_half_dt;
    sim->has_pending = info->has_pending != 0;
    sim->grid_valid = false;
    asph_status st = upload_count(sim);
    if (st != ASPH_OK) return st;
    return check_errors(sim, true);
}

asph_status asph_simulation_grid_info(asph_simulation* sim, asph_grid_info* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    for (int a = 0; a < 3; a++) {
        out->reference_cells[a] = sim->grid.gs[a];
        out->reference_cell_size[a] = sim->grid.cs[a];
        out->sub_cells[a] = sim->grid.sgs[a];
    }
    out->cell_count = sim->grid.ncells;
    out->key_bits = 3 * sim->grid.bits;
    CK(cudaStreamSynchronize(sim->stream));
    uint32_t ex[2];
    CK(cudaMemcpy(ex, sim->ex, sizeof(ex), cudaMemcpyDeviceToHost));
    out->excluded_cells[0] = ex[0];
    out->excluded_cells[1] = ex[1];
    out->boundary_excluded_cells[0] = sim->bex[0];
    out->boundary_excluded_cells[1] = sim->bex[1];
    return ASPH_OK;
}

asph_status asph_simulation_read_grid(asph_simulation* sim, uint32_t* keys, uint32_t key_capacity,
                                      uint32_t* cell_start, uint32_t* cell_end, uint32_t cell_capacity) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    CK(cudaStreamSynchronize(sim->stream));
    if (keys) {
        if (key_capacity < sim->n) return fail(ASPH_ERR_CAPACITY, "keys array too small");
        if (sim->n) CK(cudaMemcpy(keys, sim->keys, sizeof(uint32_t) * sim->n, cudaMemcpyDeviceToHost));
    }
    if (cell_start || cell_end) {
        if (cell_capacity < sim->grid.ncells) return fail(ASPH_ERR_CAPACITY, "cell arrays too small");
        if (cell_start)
            CK(cudaMemcpy(cell_start, sim->cell_start, sizeof(uint32_t) * sim->grid.ncells, cudaMemcpyDeviceToHost));
        if (cell_end)
            CK(cudaMemcpy(cell_end, sim->cell_end, sizeof(uint32_t) * sim->grid.ncells, cudaMemcpyDeviceToHost));
    }
    return ASPH_OK;
}

asph_status asph_simulation_last_refinement(asph_simulation* sim, asph_refinement_report* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = sim->last_report;
    return ASPH_OK;
}

asph_status asph_simulation_enable_timing(asph_simulation* sim, int enable) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    CK(cudaStreamSynchronize(sim->stream));
    (void)sim->harvest();
    for (int k = 0; k < (int)ASPH_KERNEL_COUNT; k++) {
        sim->ms[k] = 0.0;
        sim->timed[k] = 0;
    }
    sim->timing = enable != 0;
    return ASPH_OK;
}

asph_status asph_simulation_kernel_times(asph_simulation* sim, double* ms, uint32_t* launches, uint32_t n) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    CK(cudaStreamSynchronize(sim->stream));
    const cudaError_t he = sim->harvest();
    if (he != cudaSuccess) return cuda_fail(he, "cudaEventElapsedTime");
    for (uint32_t k = 0; k < n && k < ASPH_KERNEL_COUNT; k++) {
        if (ms) ms[k] = sim->ms[k];
        if (launches) launches[k] = sim->timed[k];
    }
    return ASPH_OK;
}

asph_status asph_simulation_launch_count(const asph_simulation* sim, uint64_t* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = sim->launches;
    return ASPH_OK;
}

}  // extern "C"

// Records the ids of merged and split particles of each refinement pass (test hook, not in asph.h).
extern "C" asph_status asph_debug_record_refinement(asph_simulation* sim, int enable) {
    API_ENTRY();
    if (!sim) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation");
    if (enable && !sim->dbg_ids) {
        asph_status st = dalloc(sim->dbg_ids, 3 * (size_t)sim->cap);
        if (st != ASPH_OK) return st;
    }
    sim->record_ids = enable != 0 && sim->adaptive;
    return ASPH_OK;
}

extern "C" asph_status asph_debug_refinement_ids(asph_simulation* sim, uint32_t* keep, uint32_t* removed,
                                                 uint32_t* split, uint32_t capacity) {
    API_ENTRY();
    if (!sim || !sim->dbg_ids) return fail(ASPH_ERR_INVALID_ARGUMENT, "recording not enabled");
    CK(cudaStreamSynchronize(sim->stream));
    const uint32_t np = sim->last_pairs_listed, ns = sim->last_splits_listed;
    if (capacity < np || capacity < ns) return fail(ASPH_ERR_CAPACITY, "arrays too small");
    if (keep && np) CK(cudaMemcpy(keep, sim->dbg_ids, 4 * (size_t)np, cudaMemcpyDeviceToHost));
    if (removed && np) CK(cudaMemcpy(removed, sim->dbg_ids + sim->cap, 4 * (size_t)np, cudaMemcpyDeviceToHost));
    if (split && ns) CK(cudaMemcpy(split, sim->dbg_ids + 2 * (size_t)sim->cap, 4 * (size_t)ns, cudaMemcpyDeviceToHost));
    return ASPH_OK;
}

// ------------------------------------------------------------------------------------------------ no-alloc sort
// asph_grid_sort_noalloc: the cell-key sort with its scratch in one fixed device array instead of cudaMalloc.
// Callers that cannot allocate: hosts that own all device memory through their own allocator (a renderer that
// imports its particle buffers under a fixed budget) and frame loops in which cudaMalloc/cudaFree would stall
// other streams (cudaFree synchronises the device) or could fail mid-frame. Nothing here allocates: no
// cudaMalloc/cudaFree, no allocating library. The scratch is shared by every call on a device, so calls that
// may overlap race on it; the caller serialises them.

namespace {
constexpr uint32_t kNoAllocMax = ASPH_NOALLOC_MAX_PARTICLES;
constexpr size_t kNoAllocTiles = (kNoAllocMax + kSortTile - 1) / kSortTile + 1;
// the layout of sort_scratch_bytes(kNoAllocMax): ping-pong keys and values, digit counts, tile counters, look-back
constexpr size_t kNoAllocSortBytes =
    sizeof(uint32_t) * ((size_t)2 * kNoAllocMax + 4 * 256 + 4 + (size_t)4 * kNoAllocTiles * 256) + 256;
constexpr size_t kNoAllocHead = 256;  // word 0: the particle count read by the sort kernels
constexpr int kNoAllocMaxDevices = 64;
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocHead + kNoAllocSortBytes];

namespace {

std::mutex g_noalloc_mutex;
void* g_noalloc_base[kNoAllocMaxDevices] = {};

// Sub-cell keys of the caller's positions (the key of k_keys), identity values, and the count for the sort.
__global__ void __launch_bounds__(256) k_noalloc_keys(GridDev g, const float4* __restrict__ pos, uint32_t n,
                                                      uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                      uint32_t* d_n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *d_n = n;
    if (i >= n) return;
    const float4 p = pos[i];
    uint32_t key, refkey;
    cell_of(g, p.x, p.y, p.z, key, refkey);
    keys[i] = key;
    vals[i] = i;
}

// Scratch address on the current device. It is looked up again on every call made outside stream capture (the
// lookup is cheap), so a device reset or a re-created primary context between calls finds the array's new address;
// a call inside a capture uses the address of the last call outside one, which is why the first call on a device
// must come before any capture.
asph_status noalloc_base(cudaStream_t stream, void** out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(ASPH_ERR_UNSUPPORTED, "device ordinal out of range");
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(stream, &cs));
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (cs == cudaStreamCaptureStatusNone) {
        CK(cudaGetSymbolAddress(&g_noalloc_base[dev], g_noalloc_scratch));
    } else if (g_noalloc_base[dev] == nullptr) {
        return fail(ASPH_ERR_UNSUPPORTED, "asph_grid_sort_noalloc: the first call on a device must not be captured");
    }
    *out = g_noalloc_base[dev];
    return ASPH_OK;
}

}  // namespace

extern "C" asph_status asph_grid_sort_noalloc(const asph_parameters* params, const float* positions, uint32_t count,
                                              uint32_t* sorted_keys, uint32_t* order, uint32_t* cell_start,
                                              uint32_t* cell_end, uint32_t cell_capacity, uint32_t* device_errors,
                                              void* stream) {
    API_ENTRY();
    if (!params || !device_errors) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    if (count > kNoAllocMax)
        return fail(ASPH_ERR_CAPACITY, "asph_grid_sort_noalloc: count " + std::to_string(count) +
                                           " exceeds the fixed scratch limit of " + std::to_string(kNoAllocMax) +
                                           " particles");
    if (count > 0 && (!positions || !sorted_keys || !order))
        return fail(ASPH_ERR_INVALID_ARGUMENT, "null device array");
    if ((cell_start == nullptr) != (cell_end == nullptr))
        return fail(ASPH_ERR_INVALID_ARGUMENT, "cell_start and cell_end must both be given or both be NULL");
    if (reinterpret_cast<uintptr_t>(positions) % 16 != 0)
        return fail(ASPH_ERR_INVALID_ARGUMENT, "positions must be 16-byte aligned");
    GridDev g;
    asph_status st = make_grid(*params, g);
    if (st != ASPH_OK) return st;
    if (cell_start && cell_capacity < g.ncells)
        return fail(ASPH_ERR_CAPACITY, "cell tables need " + std::to_string(g.ncells) + " entries");
    if (sort_scratch_bytes(kNoAllocMax) > kNoAllocSortBytes)
        return fail(ASPH_ERR_UNSUPPORTED, "sort scratch layout larger than the fixed array");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void* base = nullptr;
    if ((st = noalloc_base(s, &base)) != ASPH_OK) return st;
    uint32_t* d_n = static_cast<uint32_t*>(base);
    SortScratch ss;
    sort_scratch_bind(ss, static_cast<unsigned char*>(base) + kNoAllocHead, kNoAllocMax);
    if (count > 0) {
        k_noalloc_keys<<<blocks_for(count), 256, 0, s>>>(g, reinterpret_cast<const float4*>(positions), count,
                                                         sorted_keys, order, d_n);
        CK_LAUNCH("k_noalloc_keys");
        uint32_t* keys = sorted_keys;
        uint32_t* vals = order;
        radix_sort_pairs(keys, vals, d_n, count, 3 * g.bits, ss, device_errors, s);
        CK_LAUNCH("radix sort");
        if (keys != sorted_keys) {  // odd number of digit passes: the result is in the scratch half
            CK(cudaMemcpyAsync(sorted_keys, keys, sizeof(uint32_t) * count, cudaMemcpyDeviceToDevice, s));
            CK(cudaMemcpyAsync(order, vals, sizeof(uint32_t) * count, cudaMemcpyDeviceToDevice, s));
        }
    }
    if (cell_start) {
        CK(cudaMemsetAsync(cell_start, 0xff, sizeof(uint32_t) * g.ncells, s));
        CK(cudaMemsetAsync(cell_end, 0, sizeof(uint32_t) * g.ncells, s));
        if (count > 0) {
            k_cells_only<<<blocks_for(count), 256, 0, s>>>(g, sorted_keys, d_n, cell_start, cell_end);
            CK_LAUNCH("k_cells_only");
        }
    }
    return ASPH_OK;
}

// ------------------------------------------------------------------------------------------------ batches
// Independent simulations advanced together (asph_batch, and the serving loop of server.cpp). Each simulation runs
// on its own streams, so their steps overlap on the device. A plain step (no refinement pass) is captured once as
// a CUDA graph per buffer parity and replayed; its kernels read the particle count from the device, so a graph
// replays for any count up to the bound it was captured with. Steps with a refinement pass are enqueued without
// waiting for their read-back, after every simulation's plain steps up to its next refinement frame; the read-back
// is taken when the host needs the count (a capture, the next refinement pass, the end of the advance).
namespace {

// What a captured step depends on besides the device state: the grid bound, dt and the pending half-kick.
struct StepKey {
    uint32_t bound = 0;
    float dt = 0.0f, pending_half = 0.0f;
    bool has_pending = false;
    uint64_t generation = 0;  // asph_simulation::generation at capture
    bool replays(const StepKey& o, uint32_t n) const {
        return n <= bound && bound == o.bound && std::memcmp(&dt, &o.dt, 4) == 0 &&
               std::memcmp(&pending_half, &o.pending_half, 4) == 0 && has_pending == o.has_pending &&
               generation == o.generation;
    }
};

// grid bound of a captured step: room for growth by refinement without a new capture
uint32_t bound_for(const asph_simulation* s) {
    const uint64_t b = ((uint64_t)s->n + s->n / 8 + 256 + 255) / 256 * 256;
    return (uint32_t)std::min<uint64_t>(b, s->cap);
}

}  // namespace

namespace asph {

struct SceneGraph {
    cudaGraphExec_t exec[2] = {nullptr, nullptr};  // by buffer parity (asph_simulation::cur) at the step's start
    StepKey key[2];
    uint64_t launches[2] = {0, 0};                 // kernels in the captured step
};

SceneGraph* scene_graph_new() { return new (std::nothrow) SceneGraph(); }

void scene_graph_free(SceneGraph* g) {
    if (!g) return;
    for (int p = 0; p < 2; p++)
        if (g->exec[p]) cudaGraphExecDestroy(g->exec[p]);
    delete g;
}

}  // namespace asph

namespace {

void drop_graph(SceneGraph& g, int parity) {
    if (g.exec[parity]) cudaGraphExecDestroy(g.exec[parity]);
    g.exec[parity] = nullptr;
}

// Captures one plain step of s as a graph for its current parity; the simulation's host state is left as it was.
asph_status capture_step(asph_simulation* s, SceneGraph& g, float dt) {
    const int parity = s->cur;
    drop_graph(g, parity);
    const int cur = s->cur;
    const uint32_t frame = s->frame;
    const float pending_half = s->pending_half;
    const bool has_pending = s->has_pending, grid_valid = s->grid_valid, timing = s->timing;
    const uint64_t launches = s->launches;
    const uint32_t bound = bound_for(s);
    s->timing = false;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    s->graph_mode = true;
    s->grid_n = bound;
    const asph_status st = run_step(s, dt, ASPH_STAGE_ALL);
    s->graph_mode = false;
    const cudaError_t ce = cudaStreamEndCapture(s->stream, &graph);
    g.launches[parity] = s->launches - launches;
    s->cur = cur;
    s->frame = frame;
    s->pending_half = pending_half;
    s->has_pending = has_pending;
    s->grid_valid = grid_valid;
    s->timing = timing;
    s->launches = launches;
    if (st != ASPH_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    // per-node priorities: the heavy kernels keep the priority they were launched with (launch_with_priority)
    const cudaError_t ie = cudaGraphInstantiateWithFlags(&g.exec[parity], graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        g.exec[parity] = nullptr;
        return cuda_fail(ie, "cudaGraphInstantiate");
    }
    g.key[parity] = StepKey{bound, dt, s->pending_half, s->has_pending, s->generation};
    return ASPH_OK;
}

// One plain step of s from its graph (captured first if the step's inputs changed). A pending refinement
// read-back is taken only when its worst case exceeds the graph's bound.
asph_status graph_step(asph_simulation* s, SceneGraph& g, float dt, AdvanceStats& stats) {
    const int parity = s->cur;
    const StepKey key{g.key[parity].bound, dt, s->pending_half, s->has_pending, s->generation};
    const uint32_t n_max = s->refine_pending ? count_after_refine_bound(s) : s->n;
    if (!g.exec[parity] || !g.key[parity].replays(key, n_max)) {
        asph_status st = refine_finish(s);
        if (st != ASPH_OK) return st;
        if (!g.exec[parity] || !g.key[parity].replays(key, s->n)) {
            if ((st = ensure_rows(s, bound_for(s))) != ASPH_OK) return st;
            if ((st = capture_step(s, g, dt)) != ASPH_OK) return st;
            stats.captures++;
        }
    }
    CK(cudaGraphLaunch(g.exec[parity], s->stream));
    // the host-side effects of run_step on a plain step
    s->cur = 1 - s->cur;
    s->grid_valid = true;
    s->pending_half = dt / 2.0f;
    s->has_pending = true;
    s->frame++;
    s->launches += g.launches[parity];
    stats.graph_steps++;
    return ASPH_OK;
}

}  // namespace

namespace asph {

// plain steps a simulation may run ahead per round of advance_scenes (the reference's default refinement cooldown)
constexpr uint32_t kRoundSteps = 10;

asph_status advance_scenes(asph_simulation* const* sims, SceneGraph* const* graphs, const float* dts, uint32_t* left,
                           size_t count, AdvanceStats& stats) {
    for (size_t k = 0; k < count; k++) {
        if (!sims[k] || !graphs[k]) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation or graph cache");
        if (!std::isfinite(dts[k])) return fail(ASPH_ERR_INVALID_ARGUMENT, "delta time must be finite");
    }
    asph_status st;
    for (;;) {
        bool any = false;
        // queue every simulation's plain steps up to its next refinement frame, at most kRoundSteps of them, so
        // that no simulation runs far ahead of the others: the device's work queues stay mixed to the end
        for (size_t k = 0; k < count; k++) {
            asph_simulation* s = sims[k];
            for (uint32_t r = 0; r < kRoundSteps && left[k] > 0 && !refinement_due(s); r++) {
                // an empty simulation, and a first step (no pending half-kick: its graph would replay only once),
                // run eagerly
                if ((s->n == 0 || !s->has_pending) && !s->refine_pending) {
                    if ((st = run_step(s, dts[k], ASPH_STAGE_ALL)) != ASPH_OK) return st;
                } else if ((st = graph_step(s, *graphs[k], dts[k], stats)) != ASPH_OK) {
                    return st;
                }
                left[k]--;
                any = true;
            }
        }
        // then the refinement frames, enqueued without waiting for their read-backs
        for (size_t k = 0; k < count; k++) {
            if (left[k] == 0 || !refinement_due(sims[k])) continue;
            asph_simulation* s = sims[k];
            if ((st = refine_finish(s)) != ASPH_OK) return st;  // a pass starts from the previous one's count
            if ((st = run_step(s, dts[k], ASPH_STAGE_ALL, true)) != ASPH_OK) return st;
            stats.eager_steps++;
            left[k]--;
            any = true;
        }
        if (!any) break;
    }
    for (size_t k = 0; k < count; k++)
        if ((st = refine_finish(sims[k])) != ASPH_OK) return st;
    for (size_t k = 0; k < count; k++)
        if ((st = check_errors(sims[k], true)) != ASPH_OK) return st;
    return ASPH_OK;
}

}  // namespace asph

// ------------------------------------------------------------------------------------------------ segmented batches
// A batch step in which the plain-stepping scenes of a size bucket run their density and force passes as segmented
// launches: each scene's integrate, sort and reorder on its own stream, then one launch per pass for up to
// kSegScenes scenes (persistent ordinary kernels walking a queue of 128-particle work items round robin, warp kernels
// striding over each scene's heavy and long-row queues), instead of one launch per pass and scene. The whole step
// (forks and joins included) is captured as one CUDA graph keyed by every member's step inputs and replayed.
// Scenes that refine this frame, take their first step, or sit in a bucket the tuner gave per-scene graphs step
// as in advance_scenes. Results equal the per-scene path's bit for bit: every particle is summed by the same device
// code. The autotuner times the choices (per bucket: segmented or per-scene graphs; work items per CTA turn;
// persistent CTAs per SM or one CTA per turn's items) over the batch's first plain frames and keeps the fastest.
namespace {

constexpr uint32_t kBuckets = 3;  // particle counts below 16k, below 64k, and above
uint32_t bucket_of(uint32_t n) { return n < 16384u ? 0u : (n < 65536u ? 1u : 2u); }

struct SegConfig {
    uint8_t segmented[kBuckets] = {1, 1, 1};
    uint32_t chunk = 1;       // consecutive work items per CTA turn
    uint32_t ctas_per_sm = 7; // CTAs of the ordinary kernels per SM (persistent loop); 0: one per `chunk` items
    bool operator==(const SegConfig& o) const {
        return std::memcmp(segmented, o.segmented, sizeof(segmented)) == 0 && chunk == o.chunk &&
               ctas_per_sm == o.ctas_per_sm;
    }
};

struct SegGraph {
    std::vector<uint64_t> key;
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> member_launches;
    uint64_t last_use = 0;
};

constexpr size_t kSegGraphCache = 8;

}  // namespace

struct SegEngine {
    cudaStream_t main = nullptr, aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_mid = nullptr, ev_aux = nullptr, ev_done = nullptr;
    std::vector<cudaEvent_t> ev_member;
    std::vector<SegGraph> cache;
    uint64_t clock = 0;
    int priority_hi = 0;
    uint32_t sms = 0;
    SegConfig cfg;        // the configuration of the frame being stepped
    SegConfig tuned_cfg;  // the autotuner's choice
    uint32_t mode = ASPH_BATCH_AUTO;
    bool tuned = false;
    // tuner state: candidate configurations, the frame times measured for each, the candidate being timed
    std::vector<SegConfig> trials;
    std::vector<double> trial_ms;
    size_t trial = 0;
    uint32_t trial_frames = 0;
    double trial_acc = 0.0;
    uint32_t trial_phase = 0;
    std::vector<std::pair<SegConfig, double>> log;
    uint64_t seg_steps = 0, seg_captures = 0;
};

namespace {

void seg_free(SegEngine* E) {
    if (!E) return;
    for (SegGraph& g : E->cache)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (cudaEvent_t e : E->ev_member)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {E->ev_fork, E->ev_mid, E->ev_aux, E->ev_done})
        if (e) cudaEventDestroy(e);
    if (E->main) cudaStreamDestroy(E->main);
    if (E->aux) cudaStreamDestroy(E->aux);
    delete E;
}

asph_status seg_new(size_t members, SegEngine*& out) {
    out = nullptr;
    SegEngine* E = new (std::nothrow) SegEngine();
    if (!E) return fail(ASPH_ERR_OUT_OF_MEMORY, "segmented batch");
    int lo = 0, hi = 0, dev = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&E->main, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&E->aux, cudaStreamNonBlocking, hi);
    E->priority_hi = hi;
    for (cudaEvent_t* ev : {&E->ev_fork, &E->ev_mid, &E->ev_aux, &E->ev_done})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    E->ev_member.assign(members, nullptr);
    for (size_t k = 0; k < members && e == cudaSuccess; k++)
        e = cudaEventCreateWithFlags(&E->ev_member[k], cudaEventDisableTiming);
    int sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    E->sms = (uint32_t)(sms > 0 ? sms : 1);
    if (e != cudaSuccess) {
        seg_free(E);
        return cuda_fail(e, "segmented batch setup");
    }
    out = E;
    return ASPH_OK;
}

// Members grouped by kernel variant (periodic box; Morris viscosity; cohesion term), at most kSegScenes a group.
struct SegGroup {
    bool periodic, morris, sigma;
    std::vector<uint32_t> members;
};

std::vector<SegGroup> seg_groups(asph_simulation* const* sims, const std::vector<uint32_t>& M) {
    std::vector<SegGroup> out;
    for (uint32_t k : M) {
        const asph_simulation* s = sims[k];
        const bool p = s->grid.periodic != 0, m = s->phys.morris != 0, g = s->phys.sigma_on != 0;
        SegGroup* hit = nullptr;
        for (SegGroup& q : out)
            if (q.periodic == p && q.morris == m && q.sigma == g && q.members.size() < kSegScenes) hit = &q;
        if (!hit) {
            out.push_back(SegGroup{p, m, g, {}});
            hit = &out.back();
        }
        hit->members.push_back(k);
    }
    return out;
}

// Enqueues one plain step of every member: their grid stages on their own streams, the segmented passes on the
// engine's streams, everything ordered after E.main's current work and joined back into E.main. The members'
// host state advances as run_step's would (cur flips in the grid stage; the caller applies the rest).
asph_status seg_enqueue(SegEngine& E, asph_simulation* const* sims, const std::vector<uint32_t>& M, const float* dts,
                        uint32_t& launches_out) {
    launches_out = 0;
    CK(cudaEventRecord(E.ev_fork, E.main));
    for (uint32_t k : M) {
        asph_simulation* s = sims[k];
        CK(cudaStreamWaitEvent(s->stream, E.ev_fork, 0));
        asph_status st = run_step(s, dts[k], ASPH_STAGE_GRID);
        if (st != ASPH_OK) return st;
        CK(cudaMemsetAsync(s->fheavy_n, 0, 4 * sizeof(uint32_t), s->stream));
        CK(cudaEventRecord(E.ev_member[k], s->stream));
        CK(cudaStreamWaitEvent(E.main, E.ev_member[k], 0));
    }
    const std::vector<SegGroup> groups = seg_groups(sims, M);
    std::vector<SegLaunch> tables(groups.size());
    for (size_t gi = 0; gi < groups.size(); gi++) {
        SegLaunch& L = tables[gi];
        std::memset(&L, 0, sizeof(L));
        L.nscenes = (uint32_t)groups[gi].members.size();
        L.chunk = E.cfg.chunk;
        uint32_t items = 0;
        for (uint32_t q = 0; q < L.nscenes; q++) {
            asph_simulation* s = sims[groups[gi].members[q]];
            L.item_start[q] = items;
            L.sc[q].a = s->args(s->cur);
            L.sc[q].c = s->cells();
            L.sc[q].b = s->boundary();
            L.sc[q].nl = s->nbrs();
            items += (s->span() + kSegItem - 1) / kSegItem;
        }
        L.item_start[L.nscenes] = items;
        L.total_items = items;
    }
    const uint32_t warp_ctas = E.sms * 2;
    // ordinary kernels: one CTA per `chunk` items, at most ctas_per_sm per SM (0: no limit)
    auto ord_ctas = [&](const SegLaunch& L) -> uint32_t {
        const uint32_t need = (L.total_items + L.chunk - 1) / L.chunk;
        const uint32_t cap = E.cfg.ctas_per_sm ? E.sms * E.cfg.ctas_per_sm : need;
        return std::max<uint32_t>(1u, std::min(need, cap));
    };
    auto pass = [&](SegPass p, cudaStream_t st, int prio, uint32_t ctas, bool ordinary) -> asph_status {
        for (size_t gi = 0; gi < groups.size(); gi++) {
            const SegLaunch& L = tables[gi];
            const cudaError_t e = launch_segmented(p, L, ordinary ? ord_ctas(L) : ctas, st, prio, groups[gi].periodic,
                                                   groups[gi].morris, groups[gi].sigma);
            if (e != cudaSuccess) return cuda_fail(e, "segmented pass");
            launches_out++;
        }
        return ASPH_OK;
    };
    asph_status st;
    // density: box-heavy particles on the high-priority stream beside the ordinary pass
    CK(cudaEventRecord(E.ev_mid, E.main));
    CK(cudaStreamWaitEvent(E.aux, E.ev_mid, 0));
    if ((st = pass(kSegDensityHeavy, E.aux, E.priority_hi, warp_ctas, false)) != ASPH_OK) return st;
    if ((st = pass(kSegDensity, E.main, 0, 0, true)) != ASPH_OK) return st;
    if ((st = pass(kSegDensityOverflow, E.main, 0, warp_ctas, false)) != ASPH_OK) return st;
    if ((st = pass(kSegDensityRow, E.main, 0, warp_ctas, false)) != ASPH_OK) return st;
    CK(cudaEventRecord(E.ev_mid, E.main));
    CK(cudaEventRecord(E.ev_aux, E.aux));
    CK(cudaStreamWaitEvent(E.main, E.ev_aux, 0));
    // forces
    CK(cudaStreamWaitEvent(E.aux, E.ev_mid, 0));
    if ((st = pass(kSegForcesHeavy, E.aux, E.priority_hi, warp_ctas, false)) != ASPH_OK) return st;
    if ((st = pass(kSegForces, E.main, 0, 0, true)) != ASPH_OK) return st;
    if ((st = pass(kSegForcesRow, E.main, 0, warp_ctas, false)) != ASPH_OK) return st;
    CK(cudaEventRecord(E.ev_aux, E.aux));
    CK(cudaStreamWaitEvent(E.main, E.ev_aux, 0));
    return ASPH_OK;
}

std::vector<uint64_t> seg_key(const SegEngine& E, asph_simulation* const* sims, const std::vector<uint32_t>& M,
                              const float* dts) {
    std::vector<uint64_t> key;
    key.reserve(M.size() * 4 + 4);
    key.push_back(((uint64_t)E.cfg.chunk << 32) | E.cfg.ctas_per_sm);
    for (uint32_t k : M) {
        const asph_simulation* s = sims[k];
        uint32_t dtb, phb;
        std::memcpy(&dtb, &dts[k], 4);
        std::memcpy(&phb, &s->pending_half, 4);
        key.push_back(s->serial);
        key.push_back(((uint64_t)k << 32) | ((uint64_t)s->cur << 1) | (s->has_pending ? 1u : 0u));
        key.push_back(((uint64_t)bound_for(s) << 32) | dtb);
        key.push_back(((uint64_t)phb << 32) | (uint32_t)(s->generation & 0xffffffffu));
    }
    return key;
}

// One plain step of the members through a cached (or newly captured) whole-step graph.
asph_status seg_step(SegEngine& E, asph_simulation* const* sims, const std::vector<uint32_t>& M, const float* dts,
                     AdvanceStats& stats) {
    // a pending refinement read-back is taken where its worst case would exceed the bound a graph is keyed with
    for (uint32_t k : M) {
        asph_simulation* s = sims[k];
        if (s->refine_pending && count_after_refine_bound(s) > bound_for(s)) {
            asph_status st = refine_finish(s);
            if (st != ASPH_OK) return st;
        }
    }
    // rows for the grid bound a capture is keyed with (growing bumps a member's generation, part of the key)
    for (uint32_t k : M) {
        asph_status st = ensure_rows(sims[k], bound_for(sims[k]));
        if (st != ASPH_OK) return st;
    }
    const std::vector<uint64_t> key = seg_key(E, sims, M, dts);
    SegGraph* hit = nullptr;
    for (SegGraph& g : E.cache)
        if (g.exec && g.key == key) hit = &g;
    if (!hit) {
        // capture: members' host state is restored afterwards, the replay below applies the step's effects
        struct Saved {
            int cur;
            uint32_t frame;
            float pending_half;
            bool has_pending, grid_valid, timing;
            uint64_t launches;
        };
        std::vector<Saved> saved;
        saved.reserve(M.size());
        for (uint32_t k : M) {
            asph_simulation* s = sims[k];
            saved.push_back(Saved{s->cur, s->frame, s->pending_half, s->has_pending, s->grid_valid, s->timing,
                                  s->launches});
            s->timing = false;
            s->graph_mode = true;
            s->grid_n = bound_for(s);
        }
        cudaGraph_t graph = nullptr;
        CK(cudaStreamBeginCapture(E.main, cudaStreamCaptureModeThreadLocal));
        uint32_t seg_launches = 0;
        const asph_status st = seg_enqueue(E, sims, M, dts, seg_launches);
        const cudaError_t ce = cudaStreamEndCapture(E.main, &graph);
        std::vector<uint64_t> member_launches;
        for (size_t q = 0; q < M.size(); q++) {
            asph_simulation* s = sims[M[q]];
            member_launches.push_back(s->launches - saved[q].launches);
            s->graph_mode = false;
            s->cur = saved[q].cur;
            s->frame = saved[q].frame;
            s->pending_half = saved[q].pending_half;
            s->has_pending = saved[q].has_pending;
            s->grid_valid = saved[q].grid_valid;
            s->timing = saved[q].timing;
            s->launches = saved[q].launches;
        }
        // the segmented launches are counted on the first member
        if (!member_launches.empty()) member_launches[0] += seg_launches;
        if (st != ASPH_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture (segmented step)");
        SegGraph* slot = nullptr;
        if (E.cache.size() < kSegGraphCache) {
            E.cache.emplace_back();
            slot = &E.cache.back();
        } else {
            slot = &E.cache[0];
            for (SegGraph& g : E.cache)
                if (g.last_use < slot->last_use) slot = &g;
            if (slot->exec) cudaGraphExecDestroy(slot->exec);
            slot->exec = nullptr;
        }
        const cudaError_t ie =
            cudaGraphInstantiateWithFlags(&slot->exec, graph, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            slot->exec = nullptr;
            return cuda_fail(ie, "cudaGraphInstantiate (segmented step)");
        }
        slot->key = key;
        slot->member_launches = member_launches;
        hit = slot;
        stats.captures++;
        E.seg_captures++;
    }
    hit->last_use = ++E.clock;
    // the members' earlier work (their own streams) comes first
    for (uint32_t k : M) {
        CK(cudaEventRecord(E.ev_member[k], sims[k]->stream));
        CK(cudaStreamWaitEvent(E.main, E.ev_member[k], 0));
    }
    CK(cudaGraphLaunch(hit->exec, E.main));
    CK(cudaEventRecord(E.ev_done, E.main));
    for (size_t q = 0; q < M.size(); q++) {
        asph_simulation* s = sims[M[q]];
        CK(cudaStreamWaitEvent(s->stream, E.ev_done, 0));
        s->cur = 1 - s->cur;
        s->grid_valid = true;
        s->pending_half = dts[M[q]] / 2.0f;
        s->has_pending = true;
        s->frame++;
        s->launches += hit->member_launches[q];
    }
    stats.graph_steps += M.size();
    E.seg_steps++;
    return ASPH_OK;
}

// The candidate configurations, tried one after another over plain frames: the bucket choices first (all
// segmented, then the largest bucket on per-scene graphs, then the two largest, then none), then the work items per
// CTA turn and the CTAs per SM with the best bucket choice so far.
void seg_plan_trials(SegEngine& E) {
    E.trials.clear();
    SegConfig c;
    E.trials.push_back(c);
    c.segmented[2] = 0;
    E.trials.push_back(c);
    c.segmented[1] = 0;
    E.trials.push_back(c);
    c.segmented[0] = 0;
    E.trials.push_back(c);
    E.trial_ms.assign(E.trials.size(), 0.0);
    E.trial = 0;
    E.trial_frames = 0;
    E.trial_acc = 0.0;
    E.trial_phase = 0;
}

}  // namespace

// Lockstep advance of a batch: every scene one frame per round.
asph_status advance_batch(asph_simulation* const* sims, SceneGraph* const* graphs, SegEngine& E, const float* dts,
                          size_t count, uint32_t steps, AdvanceStats& stats) {
    for (size_t k = 0; k < count; k++) {
        if (!sims[k] || !graphs[k]) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation or graph cache");
        if (!std::isfinite(dts[k])) return fail(ASPH_ERR_INVALID_ARGUMENT, "delta time must be finite");
    }
    if (E.mode == ASPH_BATCH_AUTO && !E.tuned && E.trials.empty()) seg_plan_trials(E);
    asph_status st;
    std::vector<uint32_t> M;
    M.reserve(count);
    for (uint32_t t = 0; t < steps; t++) {
        // which configuration this frame runs with: a trial while tuning, then the tuner's choice; segmented mode
        // puts every bucket on segmented passes (with the tuned work-item and CTA counts once known)
        const bool tuning = E.mode == ASPH_BATCH_AUTO && !E.tuned;
        if (tuning) {
            E.cfg = E.trials[E.trial];
        } else if (E.mode == ASPH_BATCH_AUTO) {
            E.cfg = E.tuned_cfg;
        } else {
            E.cfg = E.tuned ? E.tuned_cfg : SegConfig{};
            for (uint32_t q = 0; q < kBuckets; q++) E.cfg.segmented[q] = E.mode == ASPH_BATCH_SEGMENTED ? 1 : 0;
        }
        M.clear();
        // a tuning frame is timed only when every simulation steps plainly in it; it starts with the device idle
        // and ends when all of its work (per-simulation graphs and the segmented step) has finished
        bool plain_frame = true;
        for (size_t k = 0; k < count; k++) {
            const asph_simulation* s = sims[k];
            if (refinement_due(s) || s->n == 0 || !s->has_pending) plain_frame = false;
        }
        std::chrono::steady_clock::time_point t0;
        if (tuning && plain_frame) {
            CK(cudaDeviceSynchronize());
            t0 = std::chrono::steady_clock::now();
        }
        for (size_t k = 0; k < count; k++) {
            asph_simulation* s = sims[k];
            const bool seg_ok = E.cfg.segmented[bucket_of(s->n)] != 0;
            if (refinement_due(s)) {
                if ((st = refine_finish(s)) != ASPH_OK) return st;
                if ((st = run_step(s, dts[k], ASPH_STAGE_ALL, true)) != ASPH_OK) return st;
                stats.eager_steps++;
            } else if (s->n == 0 || !s->has_pending) {
                if ((st = refine_finish(s)) != ASPH_OK) return st;
                if ((st = run_step(s, dts[k], ASPH_STAGE_ALL)) != ASPH_OK) return st;
                stats.eager_steps++;
            } else if (seg_ok) {
                M.push_back((uint32_t)k);
            } else if ((st = graph_step(s, *graphs[k], dts[k], stats)) != ASPH_OK) {
                return st;
            }
        }
        if (!M.empty() && (st = seg_step(E, sims, M, dts, stats)) != ASPH_OK) return st;
        if (tuning && plain_frame) {
            CK(cudaDeviceSynchronize());
            const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            // the first frame of a configuration captures its graphs: the second is timed
            if (E.trial_frames++ >= 1) E.trial_acc += ms;
            if (E.trial_frames >= 3) {
                E.trial_ms[E.trial] = E.trial_acc / 2.0;
                E.log.emplace_back(E.trials[E.trial], E.trial_ms[E.trial]);
                E.trial_frames = 0;
                E.trial_acc = 0.0;
                if (++E.trial == E.trials.size()) {
                    size_t best = 0;
                    for (size_t q = 1; q < E.trials.size(); q++)
                        if (E.trial_ms[q] < E.trial_ms[best]) best = q;
                    const SegConfig won = E.trials[best];
                    if (E.trial_phase == 0 && (won.segmented[0] || won.segmented[1] || won.segmented[2])) {
                        // second phase: work items per fetch and CTAs per SM around the winner
                        E.trial_phase = 1;
                        E.trials.clear();
                        E.trials.push_back(won);
                        for (uint32_t ch : {2u, 4u}) {
                            SegConfig c = won;
                            c.chunk = ch;
                            E.trials.push_back(c);
                        }
                        SegConfig c = won;
                        c.ctas_per_sm = 0;  // one CTA per work item (no persistent loop)
                        E.trials.push_back(c);
                        E.trial_ms.assign(E.trials.size(), 0.0);
                        E.trial = 0;
                    } else {
                        E.tuned_cfg = won;
                        E.tuned = true;
                    }
                }
            }
        }
    }
    for (size_t k = 0; k < count; k++)
        if ((st = refine_finish(sims[k])) != ASPH_OK) return st;
    CK(cudaStreamSynchronize(E.main));
    for (size_t k = 0; k < count; k++)
        if ((st = check_errors(sims[k], true)) != ASPH_OK) return st;
    return ASPH_OK;
}

struct asph_batch {
    std::vector<asph_simulation*> sims;
    std::vector<SceneGraph*> graphs;
    AdvanceStats stats;
    SegEngine* seg = nullptr;
};

extern "C" {

asph_status asph_batch_create(asph_simulation* const* sims, uint32_t count, asph_batch** out) {
    API_ENTRY();
    if (!out || (count > 0 && !sims)) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    for (uint32_t k = 0; k < count; k++) {
        if (!sims[k]) return fail(ASPH_ERR_INVALID_ARGUMENT, "null simulation in batch");
        if (sims[k]->stream == nullptr)
            return fail(ASPH_ERR_INVALID_ARGUMENT, "a batched simulation needs its own stream, not the default one");
        for (uint32_t q = 0; q < k; q++)
            if (sims[q] == sims[k]) return fail(ASPH_ERR_INVALID_ARGUMENT, "simulation listed twice");
    }
    asph_batch* b = new (std::nothrow) asph_batch();
    if (!b) return fail(ASPH_ERR_OUT_OF_MEMORY, "batch");
    b->sims.assign(sims, sims + count);
    {
        asph_status st = seg_new(count, b->seg);
        if (st != ASPH_OK) {
            asph_batch_destroy(b);
            return st;
        }
    }
    for (uint32_t k = 0; k < count; k++) {
        SceneGraph* g = scene_graph_new();
        if (!g) {
            asph_batch_destroy(b);
            return fail(ASPH_ERR_OUT_OF_MEMORY, "batch");
        }
        b->graphs.push_back(g);
    }
    *out = b;
    return ASPH_OK;
}

void asph_batch_destroy(asph_batch* b) {
    if (!b) return;
    for (SceneGraph* g : b->graphs) scene_graph_free(g);
    seg_free(b->seg);
    delete b;
}

asph_status asph_batch_step(asph_batch* b, const float* dts, uint32_t steps) {
    API_ENTRY();
    if (!b || (!b->sims.empty() && !dts)) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    return advance_batch(b->sims.data(), b->graphs.data(), *b->seg, dts, b->sims.size(), steps, b->stats);
}

asph_status asph_batch_set_mode(asph_batch* b, uint32_t mode) {
    API_ENTRY();
    if (!b) return fail(ASPH_ERR_INVALID_ARGUMENT, "null batch");
    if (mode != ASPH_BATCH_AUTO && mode != ASPH_BATCH_GRAPHS && mode != ASPH_BATCH_SEGMENTED)
        return fail(ASPH_ERR_INVALID_ARGUMENT, "unknown batch mode");
    b->seg->mode = mode;
    return ASPH_OK;
}

asph_status asph_batch_tuning(const asph_batch* b, asph_batch_tuning_info* out) {
    API_ENTRY();
    if (!b || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    const SegEngine& E = *b->seg;
    std::memset(out, 0, sizeof(*out));
    out->mode = E.mode;
    out->tuned = E.tuned ? 1u : 0u;
    const SegConfig& c0 = E.tuned ? E.tuned_cfg : E.cfg;
    for (uint32_t q = 0; q < kBuckets; q++) out->segmented[q] = c0.segmented[q];
    out->chunk = c0.chunk;
    out->ctas_per_sm = c0.ctas_per_sm;
    out->segmented_steps = E.seg_steps;
    out->segmented_captures = E.seg_captures;
    out->trials = (uint32_t)std::min<size_t>(E.log.size(), ASPH_BATCH_MAX_TRIALS);
    for (uint32_t q = 0; q < out->trials; q++) {
        const SegConfig& c = E.log[q].first;
        out->trial_ms[q] = E.log[q].second;
        out->trial_config[q] = (uint32_t)c.segmented[0] | ((uint32_t)c.segmented[1] << 1) |
                               ((uint32_t)c.segmented[2] << 2) | (c.chunk << 8) | (c.ctas_per_sm << 16);
    }
    return ASPH_OK;
}

asph_status asph_batch_stats(const asph_batch* b, uint64_t* graph_steps, uint64_t* eager_steps, uint64_t* captures) {
    API_ENTRY();
    if (!b) return fail(ASPH_ERR_INVALID_ARGUMENT, "null batch");
    if (graph_steps) *graph_steps = b->stats.graph_steps;
    if (eager_steps) *eager_steps = b->stats.eager_steps;
    if (captures) *captures = b->stats.captures;
    return ASPH_OK;
}

}  // extern "C"

extern "C" {

asph_status asph_simulation_device_bytes(const asph_simulation* sim, uint64_t* out) {
    API_ENTRY();
    if (!sim || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    *out = sim->device_bytes;
    return ASPH_OK;
}

asph_status asph_estimate_device_bytes(const asph_parameters* parameters, uint32_t count, uint32_t boundary_count,
                                       const asph_refinement_parameters* refinement, uint32_t max_fluid_capacity,
                                       uint32_t max_boundary_capacity, uint64_t* out) {
    API_ENTRY();
    if (!parameters || !out) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    GridDev g;
    asph_status st = make_grid(*parameters, g);
    if (st != ASPH_OK) return st;
    const bool adaptive = refinement && refinement->enabled;
    const uint32_t cap = std::max(adaptive ? refinement->max_particle_count : std::max(max_fluid_capacity, count), 1u);
    const uint32_t sort_items = std::max(cap, std::max(boundary_count, max_boundary_capacity));
    *out = device_bytes_for(cap, sort_items, g.ncells, (uint32_t)(g.gs[0] * g.gs[1] * g.gs[2]), boundary_count,
                            adaptive);
    return ASPH_OK;
}

}  // extern "C"

// Creation reads the caller's positions and boundary records in place where the device reads host memory through
// the host's page tables; 0 makes it stage them through copies as on other hosts, so that both paths can be
// compared on one device (test hook, not in asph.h). Returns the previous setting.
extern "C" int asph_debug_host_reads_in_place(int enable) {
    return g_host_reads_in_place.exchange(enable ? 1 : 0);
}

// Failure detection without a fault (test hook, not in asph.h): runs a sort pass whose bounded look-back wait runs
// out, and returns the error word it left (ASPH_DEVERR_SPIN_LIMIT expected); the context stays usable.
extern "C" asph_status asph_debug_wait_limit_probe(uint32_t* error_word) {
    API_ENTRY();
    if (!error_word) return fail(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    uint32_t* err = nullptr;
    CK(cudaMalloc(&err, sizeof(uint32_t)));
    cudaError_t e = cudaMemset(err, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = radix_sort_wait_probe(err, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(error_word, err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(err);
    if (e != cudaSuccess) return cuda_fail(e, "wait-limit probe");
    return ASPH_OK;
}
