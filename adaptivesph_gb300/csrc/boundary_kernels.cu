// boundary_kernels.cu — StaticBoundaryDomain::generate on the GPU (cuda/src/simulation/physics/StaticBoundaryDomain.cu:
// 76-174; the reference runs it on the host with a nanoflann KD-tree): the wall lattice and psi of every wall
// particle, bit-identical to the host code of boundary_domain.cpp.
//
// The lattice: six faces of the domain box widened by 0.05 m, face order bottom, top, -x, +x, -z, +z. Each face is the
// outer product of two coordinate sequences that the reference lays out with float loops (x = min; x < max;
// x += spacing); those sequences (a few hundred values) are formed on the host by the same loops, and a thread per
// wall particle reads its two coordinates from them.
//
// psi_b = rho0 / sum_{b'} W(|x_b - x_b'|, h) over the walls with |d|^2 < (2h)^2, self included, W in the reference's
// operation order (WendlandKernel.cuh:39-52). The host code sums the neighbours in ascending index order; here a thread
// walks the faces in order and, on each face, the lattice rows and columns within reach in ascending order, which is
// ascending index order too (index = face offset + row * row length + column), so the sums are the same bits. Rows
// and columns within reach come from a binary search of the sorted coordinate sequences, widened by a margin; the
// exact test |d|^2 < (2h)^2 decides. A face whose fixed coordinate is 2h or more away is skipped: then
// |d|^2 >= (2h)^2 holds in float as well (rounding is monotonic and the other terms are non-negative).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "asph_kernels.cuh"
#include "boundary_internal.h"

namespace asph {

namespace {

asph_status fail(asph_status s, const std::string& msg) { return report_error(s, msg); }
asph_status cuda_fail(cudaError_t e, const char* what) { return report_cuda_error(e, what); }

constexpr int kFaces = 6;

struct Face {
    uint32_t off;         // index of the face's first particle
    uint32_t rows, cols;  // lattice: rows of the outer sequence, columns of the inner one
    const float* outer;   // device sequences
    const float* inner;
    int axis_fixed, axis_outer, axis_inner;
    float fixed;
};

struct Lattice {
    Face face[kFaces];
    uint32_t n;
};

// the reference's float loop: v = start; v < end; v += step
void sequence(float start, float end, float step, std::vector<float>& out) {
    out.clear();
    for (float v = start; v < end; v += step) out.push_back(v);
}

__device__ __forceinline__ float wall_wendland(float r, float h) {
    // WendlandKernel.cuh:39-52 in its own operation order (as the host code evaluates it)
    const float pi = 3.141592653589793f;
    const float q = r / h;
    if (q > 2.0f) return 0.0f;
    const float h3 = (h * h) * h;
    const float t = 1.0f - 0.5f * q;
    const float t4 = (t * t) * (t * t);
    return ((21.0f / (16.0f * pi)) / h3) * t4 * (2.0f * q + 1.0f);
}

__device__ __forceinline__ void face_of(const Lattice& L, uint32_t i, int& f, uint32_t& row, uint32_t& col) {
    f = 0;
#pragma unroll
    for (int k = 1; k < kFaces; k++)
        if (i >= L.face[k].off) f = k;
    const uint32_t local = i - L.face[f].off;
    row = local / L.face[f].cols;
    col = local - row * L.face[f].cols;
}

// first index with seq[k] >= v (k = len when none)
__device__ __forceinline__ uint32_t lower_bound(const float* seq, uint32_t len, float v) {
    uint32_t lo = 0, hi = len;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(seq + mid) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(256) k_wall_positions(Lattice L, float4* pos) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.n) return;
    int f;
    uint32_t row, col;
    face_of(L, i, f, row, col);
    const Face& F = L.face[f];
    float p[3];
    p[F.axis_fixed] = F.fixed;
    p[F.axis_outer] = __ldg(F.outer + row);
    p[F.axis_inner] = __ldg(F.inner + col);
    pos[i] = make_float4(p[0], p[1], p[2], 0.0f);
}

__global__ void __launch_bounds__(256) k_wall_psi(Lattice L, const float4* __restrict__ pos, float h, float rho0,
                                                  float* __restrict__ psi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.n) return;
    const float4 pi = pos[i];
    const float p[3] = {pi.x, pi.y, pi.z};
    const float R = 2.0f * h;
    const float R2 = R * R;
    const float reach = R * 1.001f;  // search window; the exact test below decides
    float sum = 0.0f;
    for (int f = 0; f < kFaces; f++) {
        const Face& F = L.face[f];
        if (F.rows == 0 || F.cols == 0) continue;
        const float df = p[F.axis_fixed] - F.fixed;
        if (df * df >= R2) continue;
        const float po = p[F.axis_outer], pn = p[F.axis_inner];
        const uint32_t r0 = lower_bound(F.outer, F.rows, po - reach);
        const uint32_t c0 = lower_bound(F.inner, F.cols, pn - reach);
        for (uint32_t r = r0; r < F.rows && __ldg(F.outer + r) <= po + reach; r++) {
            const uint32_t base = F.off + r * F.cols;
            for (uint32_t c = c0; c < F.cols && __ldg(F.inner + c) <= pn + reach; c++) {
                const float4 pj = __ldg(pos + base + c);
                const float dx = pi.x - pj.x;
                const float dy = pi.y - pj.y;
                const float dz = pi.z - pj.z;
                const float d2 = (dx * dx + dy * dy) + dz * dz;
                if (d2 < R2) sum += wall_wendland(sqrtf(d2), h);
            }
        }
    }
    psi[i] = rho0 * (1.0f / sum);
}

__global__ void __launch_bounds__(256) k_wall_pack(const float4* __restrict__ pos, const float* __restrict__ psi,
                                                   uint32_t n, asph_boundary_particle* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    asph_boundary_particle b;
    b.position[0] = p.x;
    b.position[1] = p.y;
    b.position[2] = p.z;
    b.position[3] = p.w;
    b.psi = psi[i];
    out[i] = b;
}

}  // namespace

// Host: the six faces' sequences and counts (the float loops of StaticBoundaryDomain.cu:88-147).
static void lattice_host(const asph_domain& d, float s, std::vector<float> seq[4], uint32_t counts[kFaces],
                         float mn[3], float mx[3]) {
    for (int a = 0; a < 3; a++) {
        mn[a] = d.min[a] - 0.05f;
        mx[a] = d.max[a] + 0.05f;
    }
    sequence(mn[0], mx[0], s, seq[0]);      // x from min: bottom and top rows
    sequence(mn[2], mx[2], s, seq[1]);      // z from min: columns of bottom, top, -x, +x
    sequence(mn[1] + s, mx[1], s, seq[2]);  // y from min + s: rows of -x, +x, columns of -z, +z
    sequence(mn[0] + s, mx[0], s, seq[3]);  // x from min + s: rows of -z, +z
    const uint32_t x0 = (uint32_t)seq[0].size(), z0 = (uint32_t)seq[1].size(), y1 = (uint32_t)seq[2].size(),
                   x1 = (uint32_t)seq[3].size();
    counts[0] = counts[1] = x0 * z0;
    counts[2] = counts[3] = y1 * z0;
    counts[4] = counts[5] = x1 * y1;
}

asph_status generate_walls_device(const asph_domain& d, float spacing, float rho0, float h, cudaStream_t stream,
                                  DeviceWalls& out) {
    out = DeviceWalls{};
    if (!(spacing > 0.0f) || !(h > 0.0f)) return fail(ASPH_ERR_INVALID_ARGUMENT, "spacing and smoothing radius must be > 0");
    for (int a = 0; a < 3; a++)
        if (!(d.max[a] > d.min[a])) return fail(ASPH_ERR_INVALID_ARGUMENT, "domain max must exceed min on every axis");
    {
        double total = 0.0, e[3];
        for (int a = 0; a < 3; a++) e[a] = (d.max[a] - d.min[a] + 0.1) / spacing + 2.0;
        total = 2.0 * (e[0] * e[2] + e[1] * e[2] + e[0] * e[1]);
        if (total > 4.0e9) return fail(ASPH_ERR_CAPACITY, "too many wall particles");
    }
    std::vector<float> seq[4];
    uint32_t counts[kFaces];
    float mn[3], mx[3];
    lattice_host(d, spacing, seq, counts, mn, mx);
    uint64_t n = 0;
    for (int f = 0; f < kFaces; f++) n += counts[f];
    if (n > 0xffffffffull) return fail(ASPH_ERR_CAPACITY, "too many wall particles");
    out.n = (uint32_t)n;
    if (n == 0) return ASPH_OK;
    const size_t nseq = seq[0].size() + seq[1].size() + seq[2].size() + seq[3].size();
    cudaError_t e = cudaMalloc(&out.seq, sizeof(float) * nseq);
    if (e == cudaSuccess) e = cudaMalloc(&out.pos, sizeof(float4) * n);
    if (e == cudaSuccess) e = cudaMalloc(&out.psi, sizeof(float) * n);
    if (e != cudaSuccess) {
        free_walls(out);
        return cuda_fail(e, "wall buffers");
    }
    std::vector<float> packed;
    packed.reserve(nseq);
    const float* dseq[4];
    for (int k = 0; k < 4; k++) {
        dseq[k] = out.seq + packed.size();
        packed.insert(packed.end(), seq[k].begin(), seq[k].end());
    }
    e = cudaMemcpyAsync(out.seq, packed.data(), sizeof(float) * nseq, cudaMemcpyHostToDevice, stream);
    Lattice L{};
    L.n = (uint32_t)n;
    // bottom (x, y = min, z), top (x, y = max, z), -x (x = min, y, z), +x, -z (x, y, z = min), +z
    const int fixed_axis[kFaces] = {1, 1, 0, 0, 2, 2};
    const int outer_axis[kFaces] = {0, 0, 1, 1, 0, 0};
    const int inner_axis[kFaces] = {2, 2, 2, 2, 1, 1};
    const float fixed_val[kFaces] = {mn[1], mx[1], mn[0], mx[0], mn[2], mx[2]};
    const int outer_seq[kFaces] = {0, 0, 2, 2, 3, 3};
    const int inner_seq[kFaces] = {1, 1, 1, 1, 2, 2};
    uint32_t off = 0;
    for (int f = 0; f < kFaces; f++) {
        Face& F = L.face[f];
        F.off = off;
        F.rows = (uint32_t)seq[outer_seq[f]].size();
        F.cols = (uint32_t)seq[inner_seq[f]].size();
        F.outer = dseq[outer_seq[f]];
        F.inner = dseq[inner_seq[f]];
        F.axis_fixed = fixed_axis[f];
        F.axis_outer = outer_axis[f];
        F.axis_inner = inner_axis[f];
        F.fixed = fixed_val[f];
        off += counts[f];
    }
    const uint32_t blocks = (out.n + 255) / 256;
    if (e == cudaSuccess) {
        k_wall_positions<<<blocks, 256, 0, stream>>>(L, out.pos);
        k_wall_psi<<<blocks, 256, 0, stream>>>(L, out.pos, h, rho0, out.psi);
        e = cudaGetLastError();
    }
    // the packed sequences must outlive the copy
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        free_walls(out);
        return cuda_fail(e, "wall generation");
    }
    out.launches = 2;
    return ASPH_OK;
}

void free_walls(DeviceWalls& w) {
    if (w.seq) cudaFree(w.seq);
    if (w.pos) cudaFree(w.pos);
    if (w.psi) cudaFree(w.psi);
    w = DeviceWalls{};
}

}  // namespace asph

extern "C" asph_status asph_boundary_generate_gpu(const asph_domain* bounds, float particle_spacing,
                                                  float fluid_rest_density, float fluid_smoothing_radius,
                                                  asph_boundary_particle* out, uint32_t capacity, uint32_t* count) {
    using namespace asph;
    (void)cudaGetLastError();  // a stale, non-sticky error of an earlier call is not this call's
    if (!bounds || !count) return report_error(ASPH_ERR_INVALID_ARGUMENT, "null argument");
    if (!out) {
        // the count alone: the host loops, no device work
        std::vector<float> seq[4];
        uint32_t counts[6];
        float mn[3], mx[3];
        if (!(particle_spacing > 0.0f) || !(fluid_smoothing_radius > 0.0f))
            return report_error(ASPH_ERR_INVALID_ARGUMENT, "spacing and smoothing radius must be > 0");
        lattice_host(*bounds, particle_spacing, seq, counts, mn, mx);
        uint64_t n = 0;
        for (int f = 0; f < 6; f++) n += counts[f];
        *count = (uint32_t)n;
        return ASPH_OK;
    }
    DeviceWalls w;
    asph_status st = generate_walls_device(*bounds, particle_spacing, fluid_rest_density, fluid_smoothing_radius,
                                           nullptr, w);
    if (st != ASPH_OK) return st;
    *count = w.n;
    if (w.n > capacity) {
        free_walls(w);
        return report_error(ASPH_ERR_CAPACITY, "more wall particles than the output holds");
    }
    if (w.n == 0) return ASPH_OK;
    asph_boundary_particle* d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_out, sizeof(asph_boundary_particle) * w.n);
    if (e == cudaSuccess) {
        k_wall_pack<<<(w.n + 255) / 256, 256>>>(w.pos, w.psi, w.n, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, sizeof(asph_boundary_particle) * w.n, cudaMemcpyDeviceToHost);
    if (d_out) cudaFree(d_out);
    free_walls(w);
    if (e != cudaSuccess) return report_cuda_error(e, "wall read-back");
    return ASPH_OK;
}
