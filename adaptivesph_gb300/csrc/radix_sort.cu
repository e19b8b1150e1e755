// radix_sort.cu — stable onesweep LSD radix sort of (uint32 key, uint32 value) pairs.
//
// Replaces thrust::sort_by_key on the cell keys (cuda/src/simulation/neighbors/NeighborGrid.cu:139-145) and on
// the refinement scores (cuda/src/algorithm/AdaptiveAlgorithm.cuh:56-131). Structure (one digit pass per 8 key
// bits, after Adinets & Merrill, "Onesweep: A Faster Least Significant Digit Radix Sort for GPUs", 2022):
//   1. one histogram kernel counts the digits of every pass at once;
//   2. one scan kernel turns the counts into per-pass digit offsets;
//   3. per pass, one onesweep kernel: each CTA takes the next tile (3072 keys) from an atomic counter, ranks its
//      keys stably per digit (warp match + per-warp counters), publishes its per-digit tile counts, looks back
//      over predecessor tiles for the exclusive prefix (decoupled look-back), and scatters.
// Stability: within a tile items are ranked in index order; tiles are ordered by index; so equal keys keep
// their input order. Every wait on a predecessor tile is bounded: after kSpinLimit polls the kernel records
// ASPH_DEVERR_SPIN_LIMIT in the error word and continues with the partial prefix (the results of that sort are
// then invalid and the host reports the error), so no kernel can hang.
#include "asph_kernels.cuh"

namespace asph {

namespace {
constexpr uint32_t kStatusAgg = 1u << 30;
constexpr uint32_t kStatusIncl = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr int kWarps = kSortThreads / 32;

__global__ void __launch_bounds__(256) k_sort_hist(const uint32_t* __restrict__ keys, const uint32_t* d_n,
                                                   int passes, uint32_t* __restrict__ hist) {
    __shared__ uint32_t s[4][256];
    for (int t = threadIdx.x; t < 4 * 256; t += blockDim.x) (&s[0][0])[t] = 0;
    __syncthreads();
    const uint32_t n = *d_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        for (int p = 0; p < passes; p++) atomicAdd(&s[p][(k >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < passes * 256; t += blockDim.x) {
        const uint32_t v = (&s[0][0])[t];
        if (v) atomicAdd(hist + t, v);
    }
}

__global__ void __launch_bounds__(256) k_sort_scan(uint32_t* hist, int passes) {
    __shared__ uint32_t warp_sums[8];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (int p = 0; p < passes; p++) {
        const uint32_t v = hist[p * 256 + t];
        uint32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[w] = x;
        __syncthreads();
        uint32_t base = 0;
        for (int k = 0; k < w; k++) base += warp_sums[k];
        hist[p * 256 + t] = base + x - v;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kSortThreads) k_sort_onesweep(const uint32_t* __restrict__ keys_in,
                                                                const uint32_t* __restrict__ vals_in,
                                                                uint32_t* __restrict__ keys_out,
                                                                uint32_t* __restrict__ vals_out, const uint32_t* d_n,
                                                                int shift, const uint32_t* __restrict__ offsets,
                                                                uint32_t* lookback, uint32_t* counter,
                                                                uint32_t* err) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_wcnt[kWarps][256];
    __shared__ uint32_t s_base[256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(counter, 1u);
    for (int t = tid; t < kWarps * 256; t += kSortThreads) (&s_wcnt[0][0])[t] = 0;
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t n = *d_n;
    const uint32_t tile_start = tile * (uint32_t)kSortTile;
    if (tile_start >= n) return;  // beyond the last tile: nobody waits on it

    uint32_t k[kSortItems], v[kSortItems], rank[kSortItems];
    uint32_t d[kSortItems];
    bool valid[kSortItems];
    const uint32_t base = tile_start + (uint32_t)warp * (32u * kSortItems) + (uint32_t)lane;
#pragma unroll
    for (int j = 0; j < kSortItems; j++) {
        const uint32_t idx = base + (uint32_t)j * 32u;
        valid[j] = idx < n;
        k[j] = valid[j] ? keys_in[idx] : 0u;
        v[j] = valid[j] ? vals_in[idx] : 0u;
        d[j] = (k[j] >> shift) & 255u;
    }
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kSortItems; j++) {
        const uint32_t vmask = __ballot_sync(0xffffffffu, valid[j]);
        if (valid[j]) {
            const uint32_t peers = __match_any_sync(vmask, d[j]);
            const uint32_t lower = __popc(peers & lt);
            const uint32_t before = s_wcnt[warp][d[j]];
            rank[j] = before + lower;
            __syncwarp(vmask);
            if (lower == 0) s_wcnt[warp][d[j]] = before + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // per digit (one thread per digit): exclusive prefix over warps and the tile's count
    {
        const int dg = tid;
        uint32_t sum = 0;
#pragma unroll
        for (int w = 0; w < kWarps; w++) {
            const uint32_t c = s_wcnt[w][dg];
            s_wcnt[w][dg] = sum;
            sum += c;
        }
        uint32_t* slot = lookback + (size_t)tile * 256u + dg;
        uint32_t excl = 0;
        if (tile == 0) {
            atomicExch(slot, kStatusIncl | sum);
        } else {
            atomicExch(slot, kStatusAgg | sum);
            int64_t p = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (p >= 0) {
                const uint32_t st = *((volatile uint32_t*)(lookback + (size_t)p * 256u + dg));
                const uint32_t status = st & ~kValueMask;
                if (status == 0u) {
                    if (++spins > kSpinLimit) {
                        atomicOr(err, 0x1u);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                excl += st & kValueMask;
                if (status == kStatusIncl) break;
                p--;
            }
            atomicExch(slot, kStatusIncl | ((excl + sum) & kValueMask));
        }
        s_base[dg] = offsets[dg] + excl;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortItems; j++) {
        if (valid[j]) {
            const uint32_t pos = s_base[d[j]] + s_wcnt[warp][d[j]] + rank[j];
            keys_out[pos] = k[j];
            vals_out[pos] = v[j];
        }
    }
}

}  // namespace

size_t sort_scratch_bytes(uint32_t max_items) {
    const uint32_t tiles = (max_items + kSortTile - 1) / kSortTile + 1;
    return sizeof(uint32_t) * ((size_t)2 * max_items + 4 * 256 + 4 + (size_t)4 * tiles * 256) + 256;
}

void sort_scratch_bind(SortScratch& s, void* base, uint32_t max_items) {
    const uint32_t tiles = (max_items + kSortTile - 1) / kSortTile + 1;
    uint32_t* p = static_cast<uint32_t*>(base);
    s.hist = p;
    s.counters = p + 4 * 256;
    s.lookback = p + 4 * 256 + 4;
    s.keys_alt = s.lookback + (size_t)4 * tiles * 256;
    s.vals_alt = s.keys_alt + max_items;
    s.max_items = max_items;
    s.max_tiles = tiles;
}

int radix_sort_pairs(uint32_t*& keys, uint32_t*& vals, const uint32_t* d_n, uint32_t n_max, uint32_t key_bits,
                     SortScratch& s, uint32_t* err, cudaStream_t stream) {
    if (n_max == 0 || key_bits == 0) return 0;
    const int passes = (int)((key_bits + 7) / 8);
    const uint32_t tiles = (n_max + kSortTile - 1) / kSortTile;
    // hist, counters and the look-back words of all passes are contiguous
    cudaMemsetAsync(s.hist, 0, sizeof(uint32_t) * ((size_t)4 * 256 + 4 + (size_t)passes * tiles * 256), stream);
    int launches = 0;
    uint32_t hist_blocks = (n_max + 256 * 16 - 1) / (256 * 16);
    if (hist_blocks > 1024) hist_blocks = 1024;
    if (hist_blocks == 0) hist_blocks = 1;
    k_sort_hist<<<hist_blocks, 256, 0, stream>>>(keys, d_n, passes, s.hist);
    k_sort_scan<<<1, 256, 0, stream>>>(s.hist, passes);
    launches += 2;
    for (int p = 0; p < passes; p++) {
        k_sort_onesweep<<<tiles, kSortThreads, 0, stream>>>(keys, vals, s.keys_alt, s.vals_alt, d_n, 8 * p,
                                                            s.hist + 256 * p, s.lookback + (size_t)p * tiles * 256,
                                                            s.counters + p, err);
        launches++;
        uint32_t* t = keys;
        keys = s.keys_alt;
        s.keys_alt = t;
        t = vals;
        vals = s.vals_alt;
        s.vals_alt = t;
    }
    return launches;
}

// The bounded wait, made to run out: one digit pass of two tiles in which only the second tile's block runs (the
// tile counter starts at 1), so its look-back waits on a predecessor that never publishes. The block gives up after
// kSpinLimit polls, records ASPH_DEVERR_SPIN_LIMIT in err and finishes its tile (with an incomplete prefix; every
// position stays inside the arrays). Used by the failure-detection test; returns the first CUDA error.
cudaError_t radix_sort_wait_probe(uint32_t* err, cudaStream_t stream) {
    constexpr uint32_t n = 2 * kSortTile;
    uint32_t *keys = nullptr, *vals = nullptr, *keys_out = nullptr, *vals_out = nullptr, *scratch = nullptr;
    // scratch: count, digit counts of the pass, offsets, tile counter, look-back words of both tiles
    const size_t words = 1 + 4 * 256 + 1 + 2 * 256;
    cudaError_t e = cudaMalloc(&keys, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&vals, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&keys_out, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&vals_out, sizeof(uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&scratch, sizeof(uint32_t) * words);
    if (e == cudaSuccess) {
        uint32_t* d_n = scratch;
        uint32_t* hist = scratch + 1;
        uint32_t* counter = hist + 4 * 256;
        uint32_t* lookback = counter + 1;
        e = cudaMemsetAsync(keys, 0, sizeof(uint32_t) * n, stream);  // every key in digit 0
        if (e == cudaSuccess) e = cudaMemsetAsync(vals, 0, sizeof(uint32_t) * n, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * words, stream);
        const uint32_t host[2] = {n, 1u};
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_n, &host[0], sizeof(uint32_t), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(counter, &host[1], sizeof(uint32_t), cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) {
            k_sort_hist<<<1, 256, 0, stream>>>(keys, d_n, 1, hist);
            k_sort_scan<<<1, 256, 0, stream>>>(hist, 1);
            k_sort_onesweep<<<1, kSortThreads, 0, stream>>>(keys, vals, keys_out, vals_out, d_n, 0, hist, lookback,
                                                            counter, err);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    }
    cudaFree(keys);
    cudaFree(vals);
    cudaFree(keys_out);
    cudaFree(vals_out);
    cudaFree(scratch);
    return e;
}

}  // namespace asph
