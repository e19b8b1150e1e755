// asph_kernels.cuh — kernel argument blocks and kernel declarations shared by the host code.
#pragma once

#include "asph_device.cuh"

namespace asph {

// Particle arrays of the current (cell-sorted) buffer set.
struct StepArgs {
    GridDev grid;
    PhysDev phys;
    uint32_t n;            // particle count; with np set, only a bound for the grid size
    const uint32_t* np;    // particle count on the device (steps replayed from a graph), or null
    float4* ph;   // x, y, z, h
    float4* vm;   // vx, vy, vz, m
    float4* acc;  // ax, ay, az, 0
    float4* kc;   // 1/h, coef/h^3, dcoef/h^4, m
    float2* rp;   // rho, p/rho^2
    float* rad;
    uint32_t* id;
    uint32_t* err;
    float4* pq;   // x, y, z, (2h)^2: the support test's operands, written by the reorder kernel for the density scan
    float4* fr;   // rho, p/rho^2, 1/h, dcoef/h^4: a neighbour's force-pass operands, written by the density pass
};

// The step's particle count: from the device when the step is replayed from a graph (the count may have changed
// since the capture), otherwise the launch argument.
__device__ __forceinline__ uint32_t count_of(const StepArgs& a) { return a.np ? __ldg(a.np) : a.n; }

// Per-particle neighbour lists of the current step. The candidate cells are scanned in blocks of up to 32
// consecutive members of a sub-cell; row i holds one entry per block in which particle i accepted a neighbour:
// {first member index | periodic image code << 27, acceptance mask}, in the canonical candidate order, at
// ent[i * maxe + k]. Expanding the masks in order gives the accepted neighbours (self included) in canonical order.
// cnt[i] == kHeavyMark marks a particle whose query box spans more than 27 reference cells: queued in
// heavy[0, *heavy_n) by the reorder kernel for the warp density kernel. A particle with more than maxe entries
// (cnt[i] > maxe, the row overflowed) is queued in dover[0, *dover_n) by the density pass and its density summed by
// the warp density kernel too. Both kinds are queued in fheavy for the warp force kernel, which walks their cells.
// A particle with kRowHeavy < cnt[i] <= maxe entries (many neighbours) is summed over its row by one warp in both
// passes (row entry e on lane e mod 32): queued in drow by the density pass and in frow by the row density kernel.
// A box-heavy particle at heavy-queue position w < pool_slots also keeps its accepted blocks for the force pass:
// lane l of the warp that sums its density stores the blocks of its own sub-cells, in its visiting order, at
// pool[(w * 32 + l) * kPoolLaneEntries ...] with their number at pool_cnt[w * 32 + l], and cnt[i] = kPooled | w.
// If a lane has more than kPoolLaneEntries such blocks, cnt[i] = kHeavyMark and the force pass walks the cells.
constexpr uint32_t kHeavyMark = 0xffffffffu;
constexpr uint32_t kPooled = 0x80000000u;
constexpr uint32_t kBoundaryWalk = 0xffffffffu;
constexpr uint32_t kPoolLaneEntries = 32;
constexpr uint32_t kPoolSlots = 8192;
constexpr uint32_t kListEntries = 128;  // entries per row
constexpr uint32_t kRowHeavy = 96;      // rows longer than this are summed by a warp
struct NbrDev {
    uint2* ent;
    uint32_t* cnt;
    uint32_t* heavy;
    uint32_t* heavy_n;
    uint32_t* fheavy;
    uint32_t* fheavy_n;
    uint32_t* dover;
    uint32_t* dover_n;
    uint32_t* drow;
    uint32_t* drow_n;
    uint32_t* frow;
    uint32_t* frow_n;
    uint32_t* bcnt;  // wall entries recorded after the fluid entries of an ordinary row (kBoundaryWalk: none fit)
    uint2* pool;
    uint32_t* pool_cnt;
    uint32_t pool_slots;
    uint32_t maxe;
    uint32_t rows;  // particles the rows are allocated for: an index at or above it is flagged, not accessed
};

struct ReorderArgs {
    const uint32_t* keys_sorted;
    const uint32_t* vals_sorted;
    const float4* ph_in;
    const float4* vm_in;
    const float4* acc_in;
    const float* rad_in;
    const uint32_t* id_in;
    const float2* rp_in;  // may be null
    uint32_t* start;
    uint32_t* end;
    float* hmax;
    float* hmax_ref;
    uint32_t* heavy;    // queue of heavy particles (query box > kHeavyCells reference cells)
    uint32_t* heavy_n;
};

__global__ void k_integrate_keys(StepArgs a, float dt, float pending_half, int has_pending, uint32_t* keys,
                                 uint32_t* vals, unsigned long long* q3);
__global__ void k_keys(StepArgs a, uint32_t* keys, uint32_t* vals, unsigned long long* q3);
__global__ void k_boundary_keys(GridDev g, const float4* pos, uint32_t n, uint32_t* keys, uint32_t* vals,
                                unsigned long long* q3);
__global__ void k_excluded(const unsigned long long* q3, const uint32_t* n_ptr, uint32_t n_host, uint32_t* ex,
                           int periodic);
__global__ void k_reorder_cells(StepArgs a, ReorderArgs r);
__global__ void k_cells_only(GridDev g, const uint32_t* keys, const uint32_t* n_ptr, uint32_t* start, uint32_t* end);
__global__ void k_boundary_reorder(GridDev g, const float4* pos_in, const float* psi_in, float friction,
                                   const uint32_t* keys_sorted, const uint32_t* vals_sorted, uint32_t n,
                                   float4* pos_out, float* fric_out, uint32_t* start, uint32_t* end,
                                   uint8_t* refflag);
// density and force passes (neighbour_kernels.cu): the ordinary kernel (one thread per particle) or the heavy
// kernel (one warp per queued particle; for the density pass, over the box-heavy queue or the overflow queue)
enum DensityKernel { kDensityOrdinary, kDensityHeavy, kDensityOverflow, kDensityRow };
// `priority` (a stream priority value) is given to the heavy kernels' launches themselves, so that it holds when
// the step is replayed from a CUDA graph too.
cudaError_t launch_density(DensityKernel kind, uint32_t blocks, cudaStream_t stream, int priority, StepArgs a,
                           CellsDev c, BoundaryDev b, NbrDev nl);
enum ForceKernel { kForcesOrdinary, kForcesHeavy, kForcesRow };
cudaError_t launch_forces(ForceKernel kind, bool morris, uint32_t blocks, cudaStream_t stream, int priority, StepArgs a,
                          CellsDev c, BoundaryDev b, NbrDev nl);
// number of reference cells of the query box [x - R, x + R] above which a particle is heavy
constexpr int kHeavyCells = 27;

// Segmented passes: one launch runs a density or force pass for up to kSegScenes simulations (the scenes of a
// batch), from a table of their argument blocks passed by value (the launch's parameter space, read through the
// constant cache). The ordinary kernels walk a queue of work items, an item being kSegItem consecutive particles of
// one scene (items numbered scene by scene: item_start[k] .. item_start[k + 1] - 1 for scene k), each CTA taking
// `chunk` consecutive items per turn, round robin (persistent when the grid is smaller than the queue); the warp
// kernels stride over each scene's queue in turn. Every particle is summed by the same device code as in the
// single-simulation kernels, so results are the same bit for bit.
constexpr uint32_t kSegScenes = 64;
constexpr uint32_t kSegItem = 128;
struct SegScene {
    StepArgs a;
    CellsDev c;
    BoundaryDev b;
    NbrDev nl;
};
struct SegLaunch {
    uint32_t nscenes;
    uint32_t total_items;
    uint32_t chunk;
    uint32_t pad;
    uint32_t item_start[kSegScenes + 1];
    SegScene sc[kSegScenes];
};
enum SegPass { kSegDensity, kSegDensityHeavy, kSegDensityOverflow, kSegDensityRow, kSegForces, kSegForcesHeavy,
               kSegForcesRow };
// ctas: CTAs of the launch; variant flags as for the single kernels
cudaError_t launch_segmented(SegPass pass, const SegLaunch& L, uint32_t ctas, cudaStream_t stream, int priority,
                             bool periodic, bool morris, bool sigma);
__global__ void k_neighbor_counts(StepArgs a, CellsDev c, uint32_t* counts, unsigned long long* total);
__global__ void k_export(StepArgs a, float pending_half, int has_pending, float4* pos_out, float4* vel_out,
                         float* rho_out, float* rad_out, uint32_t* id_out);
// fixed-order reductions: kRedBlocks blocks of 256 threads write one row of kRedCols partials each, which
// k_reduce_rows combines in a fixed order (bit-identical results from run to run)
constexpr uint32_t kRedBlocks = 304;
constexpr uint32_t kRedCols = 8;
__global__ void k_totals(StepArgs a, float pending_half, int has_pending, double* rows);
__global__ void k_density_info(StepArgs a, float threshold, float rest, double* rows);
__global__ void k_reduce_rows(const double* rows, uint32_t nrows, uint32_t ncols, uint32_t min_mask, uint32_t max_mask,
                              double* out);

// ------------------------------------------------------------------ radix sort (radix_sort.cu)
// Stable LSD radix sort of (uint32 key, uint32 value) pairs, 8-bit digits, one onesweep pass per digit with
// decoupled look-back. The item count is read from device memory so a sort can follow a device-side count.
struct SortScratch {
    uint32_t* keys_alt;
    uint32_t* vals_alt;
    uint32_t* hist;      // [4][256] digit counts, then exclusive offsets
    uint32_t* lookback;  // [4][max_tiles][256]
    uint32_t* counters;  // [4] tile counters
    uint32_t max_items;
    uint32_t max_tiles;
};
constexpr int kSortThreads = 256;
constexpr int kSortItems = 12;
constexpr int kSortTile = kSortThreads * kSortItems;
size_t sort_scratch_bytes(uint32_t max_items);
void sort_scratch_bind(SortScratch& s, void* base, uint32_t max_items);
// Sorts keys/vals[0, *d_n) by bits [0, key_bits); n_max bounds *d_n. The result is in keys/vals (the
// ping-pong buffers are swapped back if the number of passes is odd). Returns the number of kernels launched.
int radix_sort_pairs(uint32_t*& keys, uint32_t*& vals, const uint32_t* d_n, uint32_t n_max, uint32_t key_bits,
                     SortScratch& s, uint32_t* err, cudaStream_t stream);
// A digit pass whose look-back wait runs out on purpose (failure-detection test); see radix_sort.cu.
cudaError_t radix_sort_wait_probe(uint32_t* err, cudaStream_t stream);

}  // namespace asph
