// asph_refine.cuh — argument block, device counters and kernels of the refinement pass.
#pragma once

#include "asph_kernels.cuh"

namespace asph {

// Device counters of one refinement pass (one uint32 each, read back once at the end of the pass).
enum RefineCounter : int {
    kCtrPositive = 0,   // merge scores > 0
    kCtrEligible,       // eligibleCount
    kCtrSortN,          // item count of the current selection sort (0 skips it)
    kCtrPairs,          // mergeCount
    kCtrPairSlot,       // slot counter for the optional id lists
    kCtrCount2,         // count after compaction
    kCtrRemoved,        // removed by compaction
    kCtrPositive2,      // split scores > 0
    kCtrSplitCand,      // particlesSplitCount on the device
    kCtrSplitBudget,    // min(candidates, removed/12)
    kCtrSplits,         // parents split
    kCtrCountOut,       // final count
    kCtrNextId,         // next free particle id
    kCtrMergeHeavy,     // merge candidates with query boxes of more than 27 reference cells (warp kernel)
    kCtrNum
};

struct RefineArgs {
    float* score;
    uint32_t* cand;
    uint32_t* flag;
    uint32_t* ctr;
    unsigned long long* slot0;  // (id << 32 | index) of the particle in the reference's slot 0
    uint32_t* keep_ids;         // optional lists for tests (may be null)
    uint32_t* removed_ids;
    uint32_t* split_ids;
    uint32_t* mqueue;  // [cap] merge candidates for the warp kernel
    uint32_t* err;
    float min_mass, max_mass, max_batch_ratio;
    float eps, alpha, center_ratio, vertex_ratio;
    float vel_split, vel_merge, vort_split, vort_merge, iface_split, iface_merge;
    float fs_split, fs_merge;  // free-surface criterion: neighbour-count deficit thresholds
    float r0, m0, rho0;
    uint32_t criterion;
};

__device__ float cbrt_newton(float x);

__global__ void k_merge_score(StepArgs a, CellsDev c, RefineArgs r);
__global__ void k_split_score(StepArgs a, CellsDev c, RefineArgs r);
__global__ void k_select_ids(StepArgs a, const uint32_t* n_ptr, uint32_t* keys, uint32_t* vals);
__global__ void k_select_split_ids(StepArgs a, RefineArgs r, uint32_t* keys, uint32_t* vals);
__global__ void k_select_scores(const float* score, const uint32_t* n_ptr, int descending, const uint32_t* vals_by_id,
                                uint32_t* keys);
__global__ void k_merge_limits(RefineArgs r, uint32_t n);
__global__ void k_cand_init(RefineArgs r, uint32_t n);
__global__ void k_merge_candidates_heavy(StepArgs a, CellsDev c, RefineArgs r);
__global__ void k_mark_eligible(RefineArgs r, const uint32_t* sel);
__global__ void k_merge_candidates(StepArgs a, CellsDev c, RefineArgs r);
__global__ void k_merge_pairs(StepArgs a, RefineArgs r);
__global__ void k_compact_count(const uint32_t* flag, uint32_t n, uint32_t* block_counts);
__global__ void k_compact_scan(uint32_t* block_counts, uint32_t nblocks, uint32_t n, RefineArgs r);
__global__ void k_compact_scatter(StepArgs a, StepArgs out, const uint32_t* flag, const uint32_t* block_offsets,
                                  const uint32_t* keys_in, uint32_t* keys_out);
__global__ void k_split_limits(RefineArgs r, uint32_t cap, uint32_t tpb);
__global__ void k_split_apply(StepArgs a, RefineArgs r, const uint32_t* sel);
__global__ void k_refine_finish(RefineArgs r);

}  // namespace asph
