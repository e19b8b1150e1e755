// refine_kernels.cu — the adaptive refinement pass (Vacondio-style split/merge) on the GPU.
//
// Follows performAdaptiveRefinement (cuda/src/simulation/AdaptiveSphSimulation.cu:102-252) and the kernels of
// cuda/src/algorithm/AdaptiveAlgorithm.cu, with every decision made deterministically:
//   * selection: stable order of (score, slot) — here (score, id) — ascending for merge, descending for split
//     (AdaptiveAlgorithm.cuh:56-131), by two stable radix sorts (id, then score);
//   * merge candidates: nearest neighbour, exact ties to the smaller id (AdaptiveAlgorithm.cu:159-206);
//   * pairs: mutual candidates, lower id keeps; non-eligible particles keep the reset candidate "slot 0"
//     (AdaptiveAlgorithm.cu:208-234, AdaptiveSphSimulation.cu:115-133); merge fused into the pair pass since
//     a keep particle is touched by exactly one pair (AdaptiveAlgorithm.cu:236-275);
//   * compaction: stable, out of place, by a block scan (replaces the racy in-place compactParticles,
//     AdaptiveAlgorithm.cu:119-157);
//   * split slots: daughters of the r-th split parent at count + 12 r, ids next_id + 12 r + k, instead of
//     atomicAdd order (AdaptiveAlgorithm.cu:69-117). The split count keeps the reference's launch shape:
//     the kernel guard uses the uncapped candidate count over ceil(budget / threadsPerBlock) blocks
//     (AdaptiveSphSimulation.cu:178-190).
// All counts stay on the device; the host reads them back once at the end of the pass.
#include "asph_kernels.cuh"
#include "asph_refine.cuh"

namespace asph {

__device__ float cbrt_newton(float xf) {
    // Newton-Raphson on y^3 = a in double: a = m 2^r in [0.5, 4) from frexp, six steps from y = 1, then scale.
    if (xf == 0.0f || isnan(xf) || isinf(xf)) return xf;
    const bool neg = xf < 0.0f;
    const double x = neg ? -(double)xf : (double)xf;
    int e;
    const double m = frexp(x, &e);
    const int k = e >= 0 ? e / 3 : -((-e + 2) / 3);
    const int r = e - 3 * k;
    const double a = ldexp(m, r);
    double y = 1.0;
#pragma unroll 1
    for (int it = 0; it < 6; it++) y = ((y + y) + a / (y * y)) / 3.0;
    y = ldexp(y, k);
    const float out = (float)y;
    return neg ? -out : out;
}

namespace {

__device__ __forceinline__ uint32_t sortable(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ void warp_count(bool pred, uint32_t* counter) {
    const unsigned b = __ballot_sync(0xffffffffu, pred);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(counter, (uint32_t)__popc(b));
}

// checkIfParticleCanBeSplitInsideDomain (cuda/src/simulation/refinement/criteria/Common.cuh:6-20)
__device__ __forceinline__ bool inside_domain(const GridDev& g, float4 p, float eps) {
    const float mo = eps * p.w;
    return !(p.x - mo < g.dmin[0] || p.x + mo > g.dmax[0] || p.y - mo < g.dmin[1] || p.y + mo > g.dmax[1] ||
             p.z - mo < g.dmin[2] || p.z + mo > g.dmax[2]);
}

// Velocity-gradient sum of the vorticity criterion (VorticityCriterion.cuh:198-229), search radius h_i.
template <bool kCull>
__device__ float vorticity_mag(const StepArgs& a, const CellsDev& c, uint32_t i) {
    const float4 pi = a.ph[i];
    const float4 vi = a.vm[i];
    const float hi = pi.w;
    float invh, wc, dwc;
    kernel_consts(hi, invh, wc, dwc);
    float d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int valid = 0;
    for_each_cell<kCull>(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], pi.x, pi.y, pi.z, hi, hi,
                         [&](uint32_t jb, uint32_t je, float, float, float) {
                             for (uint32_t j = jb; j < je; ++j) {
                                 if (j == i) continue;
                                 const float4 pj = a.ph[j];
                                 const float rx = pj.x - pi.x, ry = pj.y - pi.y, rz = pj.z - pi.z;
                                 const float dist = sqrtf(dist2(rx, ry, rz));
                                 if (dist < hi && dist > 1e-6f) {
                                     const float4 vj = a.vm[j];
                                     const float vd[3] = {vj.x - vi.x, vj.y - vi.y, vj.z - vi.z};
                                     const float gw = kernel_dw(dist, invh, dwc);
                                     const float w = vj.w / a.rp[j].x;
                                     const float gd[3] = {rx / dist, ry / dist, rz / dist};
#pragma unroll
                                     for (int p = 0; p < 3; p++)
#pragma unroll
                                         for (int q = 0; q < 3; q++) d[3 * p + q] = fmaf((w * vd[p]) * gd[q], gw, d[3 * p + q]);
                                     valid++;
                                 }
                             }
                         });
    if (valid < 4) return -1.0f;
    const float ox = d[7] - d[5], oy = d[2] - d[6], oz = d[3] - d[1];
    return sqrtf(fmaf(oz, oz, fmaf(oy, oy, ox * ox)));
}

// Neighbour-count deficit of the free-surface criterion (no reference counterpart): N = #{j != i : r^2 <= (2 h_j)^2}
// over the candidate cells of [x - 2h_i, x + 2h_i] (the per-particle count of sumAllNeighbors, Algorithm.cu:234-268)
// against N_ref = (4 pi / 3) (2 h_i)^3 rho0 / m_i - 1, the count a uniform medium of the particle's own volume gives;
// returns 1 - N / N_ref (positive where neighbours are missing: at the free surface).
template <bool kCull>
__device__ float neighbour_deficit(const StepArgs& a, const CellsDev& c, uint32_t i, float rho0) {
    const float4 pi = a.ph[i];
    const bool periodic = a.grid.periodic;
    const float R = pi.w + pi.w;
    uint32_t cnt = 0;
    for_each_cell<kCull>(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], pi.x, pi.y, pi.z, R, 0.0f,
                         [&](uint32_t jb, uint32_t je, float shx, float shy, float shz) {
                             for (uint32_t j = jb; j < je; ++j) {
                                 if (j == i) continue;
                                 const float4 pj = __ldg(a.ph + j);
                                 const float dx = (periodic ? pj.x + shx : pj.x) - pi.x;
                                 const float dy = (periodic ? pj.y + shy : pj.y) - pi.y;
                                 const float dz = (periodic ? pj.z + shz : pj.z) - pi.z;
                                 const float twoh = pj.w + pj.w;
                                 cnt += dist2(dx, dy, dz) <= twoh * twoh;
                             }
                         });
    const float nref = ((4.18879020478639f * ((R * R) * R)) * rho0) / a.vm[i].w - 1.0f;
    return 1.0f - (float)cnt / nref;
}

__device__ __forceinline__ void min_surface_distance(const GridDev& g, float4 p, float out[3]) {
    const float pp[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float lo = pp[a] - g.dmin[a];
        const float hi = g.dmax[a] - pp[a];
        const float m = hi < lo ? hi : lo;
        out[a] = m < 0.0f ? 0.0f : m;
    }
}

__device__ __forceinline__ float compmin3(const float v[3]) {
    float m = v[0];
    m = v[1] < m ? v[1] : m;
    m = v[2] < m ? v[2] : m;
    return m;
}

}  // namespace

// merge criterion per particle (VelocityCriterion.cuh:208-227, InterfaceCriterion.cuh:97-115,
// VorticityCriterion.cuh:248-312; free surface: neighbour_deficit); slot-0 particle (smallest id) found on the way.
__global__ void __launch_bounds__(256, 2) k_merge_score(StepArgs a, CellsDev c, RefineArgs r) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float s = -1.0f;
    uint64_t slot = ~0ull;
    if (i < a.n) {
        const float4 p = a.ph[i];
        const float4 v = a.vm[i];
        slot = ((uint64_t)a.id[i] << 32) | i;
        if (!(v.w > r.max_mass)) {
            if (r.criterion == 1u) {
                float md[3], nd[3];
                min_surface_distance(a.grid, p, md);
#pragma unroll
                for (int q = 0; q < 3; q++) nd[q] = md[q] / (r.iface_merge * (a.grid.dmax[q] - a.grid.dmin[q]));
                s = compmin3(nd) - 1.0f;
            } else if (r.criterion == 2u) {
                const float mag = vorticity_mag<true>(a, c, i);
                s = (mag >= 0.0f && mag < r.vort_merge) ? mag / r.vort_merge : -1.0f;
            } else if (r.criterion == 3u) {
                const float d = neighbour_deficit<true>(a, c, i, r.rho0);
                const float t = r.fs_merge;
                s = d <= t ? ((d > 0.0f ? d : 0.0f) + t) / (t + t) : -1.0f;
            } else {
                const float sp = sqrtf(fmaf(v.z, v.z, fmaf(v.y, v.y, v.x * v.x)));
                s = sp < r.vel_merge ? sp / r.vel_merge : -1.0f;
            }
        }
        r.score[i] = s;
    }
    warp_count(i < a.n && s > 0.0f, r.ctr + kCtrPositive);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t u = __shfl_xor_sync(0xffffffffu, slot, o);
        slot = u < slot ? u : slot;
    }
    if ((threadIdx.x & 31) == 0 && slot != ~0ull) atomicMin(r.slot0, (unsigned long long)slot);
}

// split criterion per particle of the compacted set (VelocityCriterion.cuh:180-206,
// InterfaceCriterion.cuh:69-95, VorticityCriterion.cuh:170-246)
__global__ void __launch_bounds__(256, 2) k_split_score(StepArgs a, CellsDev c, RefineArgs r) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = (r.ctr[kCtrRemoved] > 0u) ? r.ctr[kCtrCount2] : 0u;
    float s = -1.0f;
    if (i < n) {
        const float4 p = a.ph[i];
        const float4 v = a.vm[i];
        if (!(v.w < r.min_mass)) {
            if (r.criterion == 1u) {
                float md[3], nd[3];
                min_surface_distance(a.grid, p, md);
                if (!(compmin3(md) < r.eps * p.w)) {
#pragma unroll
                    for (int q = 0; q < 3; q++) nd[q] = md[q] / (r.iface_split * (a.grid.dmax[q] - a.grid.dmin[q]));
                    s = 1.0f - compmin3(nd);
                }
            } else if (inside_domain(a.grid, p, r.eps)) {
                if (r.criterion == 2u) {
                    const float mag = vorticity_mag<false>(a, c, i);
                    s = (mag >= 0.0f && mag > r.vort_split) ? mag : -1.0f;
                } else if (r.criterion == 3u) {
                    // within 2h of a domain face the clamp, not the air, truncates the support: no split there
                    float md[3];
                    min_surface_distance(a.grid, p, md);
                    if (a.grid.periodic || !(compmin3(md) < p.w + p.w)) {
                        const float d = neighbour_deficit<false>(a, c, i, r.rho0);
                        s = d >= r.fs_split ? d : -1.0f;
                    }
                } else {
                    const float sp = sqrtf(fmaf(v.z, v.z, fmaf(v.y, v.y, v.x * v.x)));
                    s = sp < r.vel_split ? -1.0f : sp;
                }
            }
        }
        r.score[i] = s;
    }
    warp_count(i < n && s > 0.0f, r.ctr + kCtrPositive2);
}

// Stage A of the selection: (id, index) pairs; stage B keys come from the scores in id order.
// The split selection's input: only the particles with a positive split score (the split parents are the first
// `splits` entries of the descending order, and splits <= the positive count), appended at kCtrSortN, which
// k_split_limits zeroes when there is anything to split; warp-aggregated appends, their order is then fixed by the
// sort by id. The first `splits` entries after the sorts are the ones a sort of all particles gives.
__global__ void __launch_bounds__(256) k_select_split_ids(StepArgs a, RefineArgs r, uint32_t* keys, uint32_t* vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = (r.ctr[kCtrSplits] > 0u) ? r.ctr[kCtrCount2] : 0u;
    const bool take = i < n && r.score[i] > 0.0f;
    const unsigned b = __ballot_sync(0xffffffffu, take);
    if (b == 0u) return;
    const int lane = (int)(threadIdx.x & 31u);
    uint32_t base = 0;
    if (lane == __ffs(b) - 1) base = atomicAdd(r.ctr + kCtrSortN, (uint32_t)__popc(b));
    base = __shfl_sync(0xffffffffu, base, __ffs(b) - 1);  // every lane of the warp is here (b is warp-uniform)
    if (take) {
        const uint32_t slot = base + (uint32_t)__popc(b & ((1u << lane) - 1u));
        keys[slot] = a.id[i];
        vals[slot] = i;
    }
}

__global__ void __launch_bounds__(256) k_select_ids(StepArgs a, const uint32_t* n_ptr, uint32_t* keys, uint32_t* vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *n_ptr) {
        keys[i] = a.id[i];
        vals[i] = i;
    }
}

__global__ void __launch_bounds__(256) k_select_scores(const float* score, const uint32_t* n_ptr, int descending,
                                                       const uint32_t* vals_by_id, uint32_t* keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < *n_ptr) {
        const uint32_t s = sortable(score[vals_by_id[i]]);
        keys[i] = descending ? ~s : s;
    }
}

// k = min(#score>0, round(N * maxBatchRatio)) (AdaptiveAlgorithm.cuh:107-118 / :446-455)
__global__ void k_merge_limits(RefineArgs r, uint32_t n) {
    const uint32_t lim = (uint32_t)roundf((float)n * r.max_batch_ratio);
    const uint32_t cp = r.ctr[kCtrPositive];
    r.ctr[kCtrEligible] = n > 1u ? (cp < lim ? cp : lim) : 0u;
    r.ctr[kCtrSortN] = r.ctr[kCtrEligible] > 0u ? n : 0u;
}

__global__ void __launch_bounds__(256) k_cand_init(RefineArgs r, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        r.cand[i] = (uint32_t)(*r.slot0 & 0xffffffffull);
        r.flag[i] = 0u;
    }
}

// Marks the selected merge candidates (the first `eligible` slots of the score-sorted ids) in cand[].
__global__ void __launch_bounds__(256) k_mark_eligible(RefineArgs r, const uint32_t* sel) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < r.ctr[kCtrEligible]) r.cand[sel[q]] = kEligible;
}

// identifyMergeCandidates (AdaptiveAlgorithm.cu:159-206) for the marked particles, taken in the cell order of the
// particle array rather than in score order, so that a warp's searches are neighbours and share their loads. Each
// particle's result depends on that particle alone.
__global__ void __launch_bounds__(256, 4) k_merge_candidates(StepArgs a, CellsDev c, RefineArgs r) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.n || r.cand[e] != kEligible) return;
    const float4 pe = a.ph[e];
    const float he = pe.w;
    if (box_cells(a.grid, pe, he) > kHeavyCells) {  // large box: one warp (k_merge_candidates_heavy)
        r.mqueue[atomicAdd(r.ctr + kCtrMergeHeavy, 1u)] = e;
        return;
    }
    float best = 3.402823466e38f;
    uint32_t bj = kNone, bid = 0xffffffffu;
    for_each_cell<true>(a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], pe.x, pe.y, pe.z, he, he,
                        [&](uint32_t jb, uint32_t je, float, float, float) {
                            for (uint32_t j = jb; j < je; ++j) {
                                if (j == e) continue;
                                const float4 pj = a.ph[j];
                                const float dx = pj.x - pe.x, dy = pj.y - pe.y, dz = pj.z - pe.z;
                                const float r2 = dist2(dx, dy, dz);
                                const float hm = pj.w < he ? pj.w : he;
                                if (r2 < hm * hm && a.vm[j].w < r.max_mass) {
                                    const uint32_t idj = a.id[j];
                                    if (r2 < best || (r2 == best && idj < bid)) {
                                        best = r2;
                                        bj = j;
                                        bid = idj;
                                    }
                                }
                            }
                        });
    r.cand[e] = bj;
}

// identifyMergeCandidates for the queued large boxes: one block of 8 warps per particle, the box's reference cells
// dealt to the warps and their sub-cells to the lanes (for_each_subcell_lane over 8 warps). The nearest candidate is
// the minimum of (r^2, id) over the accepted members, which does not depend on the visiting order, so the block's
// reduction gives the sequential scan's result.
__global__ void __launch_bounds__(256, 2) k_merge_candidates_heavy(StepArgs a, CellsDev c, RefineArgs r) {
    constexpr uint32_t kWarps = 8;
    __shared__ float s_best[kWarps];
    __shared__ uint32_t s_bj[kWarps], s_bid[kWarps];
    const int lane = threadIdx.x & 31;
    const uint32_t wi = threadIdx.x >> 5;
    const uint32_t nq = r.ctr[kCtrMergeHeavy];
    for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
        const uint32_t e = r.mqueue[q];
        const float4 pe = a.ph[e];
        const float he = pe.w;
        float best = 3.402823466e38f;
        uint32_t bj = kNone, bid = 0xffffffffu;
        for_each_subcell_lane(
            a.grid, c.start, c.end, c.hmax, c.hmax_ref, c.ex[0], c.ex[1], pe.x, pe.y, pe.z, he, he, lane,
            [&](uint32_t jb, uint32_t je, float, float, float) {
                for (uint32_t j = jb; j < je; ++j) {
                    if (j == e) continue;
                    const float4 pj = a.ph[j];
                    const float dx = pj.x - pe.x, dy = pj.y - pe.y, dz = pj.z - pe.z;
                    const float r2 = dist2(dx, dy, dz);
                    const float hm = pj.w < he ? pj.w : he;
                    if (r2 < hm * hm && a.vm[j].w < r.max_mass) {
                        const uint32_t idj = a.id[j];
                        if (r2 < best || (r2 == best && idj < bid)) {
                            best = r2;
                            bj = j;
                            bid = idj;
                        }
                    }
                }
            },
            wi, kWarps);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const uint32_t oj = __shfl_xor_sync(0xffffffffu, bj, o);
            const uint32_t oid = __shfl_xor_sync(0xffffffffu, bid, o);
            if (ob < best || (ob == best && oid < bid)) {
                best = ob;
                bj = oj;
                bid = oid;
            }
        }
        if (lane == 0) {
            s_best[wi] = best;
            s_bj[wi] = bj;
            s_bid[wi] = bid;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint32_t k = 1; k < kWarps; ++k) {
                if (s_best[k] < best || (s_best[k] == best && s_bid[k] < bid)) {
                    best = s_best[k];
                    bj = s_bj[k];
                    bid = s_bid[k];
                }
            }
            r.cand[e] = bj;
        }
        __syncthreads();
    }
}

// resolveMergePairs + performMerges + calculateMergedSmoothingLength (AdaptiveAlgorithm.cu:50-67, 208-275)
__global__ void __launch_bounds__(256) k_merge_pairs(StepArgs a, RefineArgs r) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool merged = false;
    if (i < a.n && r.ctr[kCtrEligible] > 0u) {
        const uint32_t c = r.cand[i];
        if (c != kNone && r.cand[c] == i && a.id[i] < a.id[c]) {
            merged = true;
            const float4 p1 = a.ph[i], p2 = a.ph[c];
            const float4 v1 = a.vm[i], v2 = a.vm[c];
            const float4 a1 = a.acc[i], a2 = a.acc[c];
            const float m1 = v1.w, m2 = v2.w;
            const float M = m1 + m2;
            const float npx = fmaf(m1, p1.x, m2 * p2.x) / M, npy = fmaf(m1, p1.y, m2 * p2.y) / M,
                        npz = fmaf(m1, p1.z, m2 * p2.z) / M;
            const float nvx = fmaf(m1, v1.x, m2 * v2.x) / M, nvy = fmaf(m1, v1.y, m2 * v2.y) / M,
                        nvz = fmaf(m1, v1.z, m2 * v2.z) / M;
            const float nax = fmaf(m1, a1.x, m2 * a2.x) / M, nay = fmaf(m1, a1.y, m2 * a2.y) / M,
                        naz = fmaf(m1, a1.z, m2 * a2.z) / M;
            float W[2];
            const float4 pp[2] = {p1, p2};
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const float dx = pp[k].x - npx, dy = pp[k].y - npy, dz = pp[k].z - npz;
                const float d = sqrtf(dist2(dx, dy, dz));
                float invh, wc, dwc;
                kernel_consts(pp[k].w, invh, wc, dwc);
                W[k] = kernel_w(d, invh, wc);
            }
            const float denom = fmaf(m1, W[0], m2 * W[1]);
            const float coef = (16.0f * kPi) / 21.0f;
            const float hn = cbrt_newton((coef * M) / denom);
            const float rn = r.r0 * cbrt_newton(M / r.m0);
            a.ph[i] = make_float4(npx, npy, npz, hn);
            a.vm[i] = make_float4(nvx, nvy, nvz, M);
            a.acc[i] = make_float4(nax, nay, naz, 0.0f);
            a.rad[i] = rn;
            a.rp[i] = make_float2(0.0f, a.rp[i].y);
            r.flag[c] = 1u;
            if (r.keep_ids) {
                const uint32_t slot = atomicAdd(r.ctr + kCtrPairSlot, 1u);
                r.keep_ids[slot] = a.id[i];
                r.removed_ids[slot] = a.id[c];
            }
        }
    }
    warp_count(merged, r.ctr + kCtrPairs);
}

// Stable compaction, phase 1: kept particles per block of 256.
__global__ void __launch_bounds__(256) k_compact_count(const uint32_t* flag, uint32_t n, uint32_t* block_counts) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool keep = i < n && flag[i] == 0u;
    const unsigned b = __ballot_sync(0xffffffffu, keep);
    __shared__ uint32_t s[8];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; w++) t += s[w];
        block_counts[blockIdx.x] = t;
    }
}

// Phase 2: exclusive scan of the block counts (one CTA), total -> ctr[kCtrCount2], removed -> ctr[kCtrRemoved].
__global__ void __launch_bounds__(1024) k_compact_scan(uint32_t* block_counts, uint32_t nblocks, uint32_t n,
                                                       RefineArgs r) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t base = 0; base < nblocks; base += 1024) {
        const uint32_t idx = base + threadIdx.x;
        const uint32_t v = idx < nblocks ? block_counts[idx] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[w] = x;
        __syncthreads();
        uint32_t pre = 0;
        for (int k = 0; k < w; k++) pre += warp_sums[k];
        const uint32_t c0 = carry;
        if (idx < nblocks) block_counts[idx] = c0 + pre + x - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c0 + pre + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const uint32_t kept = r.ctr[kCtrPairs] > 0u ? carry : n;
        r.ctr[kCtrCount2] = kept;
        r.ctr[kCtrRemoved] = n - kept;
    }
}

// Phase 3: gather kept particles (and their cell keys) into the other buffer set in order.
__global__ void __launch_bounds__(256) k_compact_scatter(StepArgs a, StepArgs out, const uint32_t* flag,
                                                         const uint32_t* block_offsets, const uint32_t* keys_in,
                                                         uint32_t* keys_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool keep = i < a.n && flag[i] == 0u;
    const unsigned b = __ballot_sync(0xffffffffu, keep);
    __shared__ uint32_t s[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) s[w] = __popc(b);
    __syncthreads();
    if (!keep) return;
    uint32_t pre = 0;
    for (int k = 0; k < w; k++) pre += s[k];
    const uint32_t pos = block_offsets[blockIdx.x] + pre + __popc(b & ((1u << lane) - 1u));
    out.ph[pos] = a.ph[i];
    out.vm[pos] = a.vm[i];
    out.acc[pos] = a.acc[i];
    out.rp[pos] = a.rp[i];
    out.rad[pos] = a.rad[i];
    out.id[pos] = a.id[i];
    if (keys_in) keys_out[pos] = keys_in[i];
}

// Split budget: k = min(#score>0, round(N' ratio)); budget = min(k, removed/12); the reference's kernel runs
// tid < k over ceil(budget/tpb)*tpb threads; capacity bounds the rest (AdaptiveSphSimulation.cu:167-193).
__global__ void k_split_limits(RefineArgs r, uint32_t cap, uint32_t tpb) {
    const uint32_t removed = r.ctr[kCtrRemoved];
    const uint32_t n2 = r.ctr[kCtrCount2];
    uint32_t ks = 0, budget = 0, M = 0;
    if (removed > 0u) {
        const uint32_t lim = (uint32_t)roundf((float)n2 * r.max_batch_ratio);
        const uint32_t cp = r.ctr[kCtrPositive2];
        ks = cp < lim ? cp : lim;
        budget = ks < removed / 12u ? ks : removed / 12u;
        if (budget > 0u) {
            const uint64_t launched = (uint64_t)((budget + tpb - 1u) / tpb) * tpb;
            M = (uint64_t)ks < launched ? ks : (uint32_t)launched;
        }
    }
    const uint32_t room = cap > n2 ? (cap - n2) / 12u : 0u;
    uint32_t splits = M < room ? M : room;
    if (splits < M) atomicOr(r.err, 0x4u);
    uint64_t last_id = (uint64_t)r.ctr[kCtrNextId] + 12ull * splits;
    if (last_id > 0xffffffffull) {
        atomicOr(r.err, 0x8u);
        splits = 0;
    }
    r.ctr[kCtrSplitCand] = ks;
    r.ctr[kCtrSplitBudget] = budget;
    r.ctr[kCtrSplits] = splits;
    r.ctr[kCtrSortN] = 0u;  // k_select_split_ids appends the positive-score particles
    r.ctr[kCtrCountOut] = n2 + 12u * splits;
}

// splitParticles (AdaptiveAlgorithm.cu:69-117): parent -> centre + 12 daughters on the icosahedron.
__global__ void __launch_bounds__(256) k_split_apply(StepArgs a, RefineArgs r, const uint32_t* sel) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t splits = r.ctr[kCtrSplits];
    if (q >= splits) return;
    const uint32_t n2 = r.ctr[kCtrCount2];
    const uint32_t next_id = r.ctr[kCtrNextId];
    const uint32_t p = sel[q];
    const float A = 1.6180339887498949f * 0.5257311121f, B = 0.5257311121f;
    const float ico[12][3] = {{0.0f, A, B},  {0.0f, A, -B},  {0.0f, -A, -B}, {0.0f, -A, B},
                              {B, 0.0f, A},  {-B, 0.0f, A},  {B, 0.0f, -A},  {-B, 0.0f, -A},
                              {A, B, 0.0f},  {A, -B, 0.0f},  {-A, B, 0.0f},  {-A, -B, 0.0f}};
    const float4 x = a.ph[p];
    const float4 v = a.vm[p];
    const float4 ac = a.acc[p];
    const float m = v.w, rr = a.rad[p], h = x.w;
    const float dm = m * r.vertex_ratio, cm = m * r.center_ratio;
    const float nr = rr * cbrt_newton(dm / m);
    const float nh = r.alpha * h;
    if (r.split_ids) r.split_ids[q] = a.id[p];
    a.ph[p] = make_float4(x.x, x.y, x.z, nh);
    a.vm[p] = make_float4(v.x, v.y, v.z, cm);
    a.rad[p] = rr * cbrt_newton(cm / m);
    const uint32_t base = n2 + 12u * q;
#pragma unroll 1
    for (uint32_t k = 0; k < 12; k++) {
        const uint32_t d = base + k;
        const float ox = (ico[k][0] * r.eps) * h, oy = (ico[k][1] * r.eps) * h, oz = (ico[k][2] * r.eps) * h;
        a.ph[d] = make_float4(x.x + ox, x.y + oy, x.z + oz, nh);
        a.vm[d] = make_float4(v.x, v.y, v.z, dm);
        a.acc[d] = ac;
        a.rad[d] = nr;
        a.rp[d] = make_float2(0.0f, 0.0f);
        a.id[d] = next_id + 12u * q + k;
    }
}

__global__ void k_refine_finish(RefineArgs r) {
    r.ctr[kCtrNextId] = r.ctr[kCtrNextId] + 12u * r.ctr[kCtrSplits];
}

}  // namespace asph
