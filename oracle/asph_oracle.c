/*
 * asph_oracle.c — CPU restatement of AdaptiveSph's per-step particle pipeline.
 * TEST INFRASTRUCTURE ONLY (the checker); see asph_oracle.h for scope and parity status.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fno-fast-math -shared -fPIC (oracle/build.py). Contraction must
 * stay off: the FP32 variant reproduces the CUDA kernels' explicit fmaf/mul/add sequence operation for
 * operation.
 */
#include "asph_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ threads */
void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) {
        omp_set_num_threads(n);
    }
#else
    (void)n;
#endif
}

int orc_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ grid geometry */
/* NeighborGrid::createGrid / calculateGridSize (cuda/src/simulation/neighbors/NeighborGrid.cu:108-121); cell
 * width 2 * h0 * wendlandRangeRatio (cuda/src/simulation/SphSimulation.cu:46-49). Each reference cell is split
 * into 2x2x2 sub-cells for the sort and the cell tables; the reference cells still define the candidate set. */
void orc_grid_make(const orc_params* P, orc_grid* g)
{
    const float cw = (2.0f * P->h0) * 2.0f;
    int32_t mx = 1;
    g->ncells = 1;
    for (int a = 0; a < 3; a++) {
        g->dmin[a] = P->dmin[a];
        g->dmax[a] = P->dmax[a];
        g->scale[a] = P->dmax[a] - P->dmin[a];
        int32_t gs = (int32_t)ceilf(g->scale[a] / cw);
        if (gs < 1) {
            gs = 1;
        }
        g->gs[a] = gs;
        g->cs[a] = g->scale[a] / (float)gs;
        g->sgs[a] = 2 * gs;
        if (g->sgs[a] > mx) {
            mx = g->sgs[a];
        }
        g->ncells *= (uint32_t)g->sgs[a];
    }
    uint32_t bits = 1;
    while ((1 << bits) < mx) {
        bits++;
    }
    g->bits = bits;
    g->periodic = P->periodic;
}

static uint32_t part1by2(uint32_t x)
{
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

static uint32_t compact1by2(uint32_t x)
{
    x &= 0x09249249u;
    x = (x ^ (x >> 2)) & 0x030c30c3u;
    x = (x ^ (x >> 4)) & 0x0300f00fu;
    x = (x ^ (x >> 8)) & 0xff0000ffu;
    x = (x ^ (x >> 16)) & 0x000003ffu;
    return x;
}

uint32_t orc_morton3(uint32_t x, uint32_t y, uint32_t z)
{
    return part1by2(x) | (part1by2(y) << 1) | (part1by2(z) << 2);
}

static uint32_t lin_of_key(const orc_grid* g, uint32_t key)
{
    const uint32_t x = compact1by2(key), y = compact1by2(key >> 1), z = compact1by2(key >> 2);
    return x + (uint32_t)g->sgs[0] * (y + (uint32_t)g->sgs[1] * z);
}

/* calculateCellIndex (cuda/src/simulation/neighbors/NeighborGrid.cuh:166-172) and flattenCellIndex (:174-177);
 * the sub-cell index is floor(2 f) of the same f = clamp(x - min) / cellSize, so it always lies inside the
 * reference cell floor(f). */
void orc_cell_of(const orc_grid* g, const float* p, uint32_t* key, uint32_t* refkey, uint32_t* lin)
{
    int32_t rc[3], sc[3];
    for (int a = 0; a < 3; a++) {
        const float rel = p[a] - g->dmin[a];
        float cl = rel < 0.0f ? 0.0f : rel;
        cl = cl > g->scale[a] ? g->scale[a] : cl;
        const float f = cl / g->cs[a];
        int32_t c = (int32_t)f;
        if (c > g->gs[a] - 1) {
            c = g->gs[a] - 1;
        }
        int32_t s2 = (int32_t)(f * 2.0f);
        if (s2 > g->sgs[a] - 1) {
            s2 = g->sgs[a] - 1;
        }
        rc[a] = c;
        sc[a] = s2;
    }
    if (key) {
        *key = orc_morton3((uint32_t)sc[0], (uint32_t)sc[1], (uint32_t)sc[2]);
    }
    if (refkey) {
        *refkey = (uint32_t)(rc[0] + g->gs[0] * (rc[1] + g->gs[1] * rc[2]));
    }
    if (lin) {
        *lin = (uint32_t)(sc[0] + g->sgs[0] * (sc[1] + g->sgs[1] * sc[2]));
    }
}

/* ------------------------------------------------------------------ neighbour-cell iterator */
/* forEachFluidNeighbor / forEachBoundaryNeighbor (cuda/src/simulation/neighbors/NeighborGrid.cuh:90-164): the
 * candidate cells are the reference cells overlapping [x - R, x + R] (truncated toward zero, clamped to the
 * grid), minus the cells the reference's boundary pass leaves unset. The canonical visiting order: reference
 * cells in z, y, x order; within each, its 2x2x2 sub-cells in z, y, x order; members of a sub-cell in
 * cell-sorted order. */
typedef struct orc_iter {
    const orc_grid* g;
    const uint32_t *start, *end;
    uint32_t ex0, ex1;
    int32_t lo[3], hi[3], r[3]; /* reference-cell box and the current reference cell (unwrapped) */
    int32_t c[3];               /* current reference cell, wrapped */
    float sh[3];                /* its periodic image offset */
    int q;                      /* next sub-cell of the current reference cell, 0..8 */
    int empty;
    uint32_t t; /* canonical index in the box of the sub-cell it_next returned: 8 * (reference cell in z, y, x
                   order within the box) + sub-cell; a heavy particle's sub-cell t is summed on lane t mod 32 */
} orc_iter;

static float clampf(float x, float lo, float hi)
{
    x = x < lo ? lo : x;
    return x > hi ? hi : x;
}

static void it_init(orc_iter* it, const orc_grid* g, const uint32_t* start, const uint32_t* end,
                    const uint32_t ex[2], const float* p, float R)
{
    it->g = g;
    it->start = start;
    it->end = end;
    it->ex0 = ex[0];
    it->ex1 = ex[1];
    it->empty = 0;
    for (int a = 0; a < 3; a++) {
        const float rel = p[a] - g->dmin[a];
        const float lof = clampf((rel - R) / g->cs[a], -1.0e7f, 1.0e7f);
        const float hif = clampf((rel + R) / g->cs[a], -1.0e7f, 1.0e7f);
        int32_t l, h;
        if (!g->periodic) {
            l = (int32_t)lof;
            h = (int32_t)hif;
            if (l < 0) {
                l = 0;
            }
            if (h > g->gs[a] - 1) {
                h = g->gs[a] - 1;
            }
        } else {
            l = (int32_t)floorf(lof);
            h = (int32_t)floorf(hif);
            if (h - l + 1 > g->gs[a]) {
                h = l + g->gs[a] - 1;
            }
        }
        if (l > h) {
            it->empty = 1;
        }
        it->lo[a] = l;
        it->hi[a] = h;
    }
    it->r[0] = it->lo[0] - 1;
    it->r[1] = it->lo[1];
    it->r[2] = it->lo[2];
    it->q = 8;
}

/* number of reference cells in the box of p with radius R (the heavy-particle criterion) */
static int64_t box_cells(const orc_grid* g, const float* p, float R)
{
    orc_iter it;
    static const uint32_t none[2] = {ORC_NONE, ORC_NONE};
    it_init(&it, g, NULL, NULL, none, p, R);
    if (it.empty) {
        return 0;
    }
    return (int64_t)(it.hi[0] - it.lo[0] + 1) * (it.hi[1] - it.lo[1] + 1) * (it.hi[2] - it.lo[2] + 1);
}

/* moves to the next reference cell of the box that is neither excluded nor outside a periodic grid */
static int it_next_ref(orc_iter* it)
{
    const orc_grid* g = it->g;
    for (;;) {
        if (++it->r[0] > it->hi[0]) {
            it->r[0] = it->lo[0];
            if (++it->r[1] > it->hi[1]) {
                it->r[1] = it->lo[1];
                if (++it->r[2] > it->hi[2]) {
                    it->empty = 1;
                    return 0;
                }
            }
        }
        int ok = 1;
        for (int a = 0; a < 3; a++) {
            int32_t c = it->r[a];
            float sh = 0.0f;
            if (g->periodic) {
                if (c < 0) {
                    c += g->gs[a];
                    sh = -g->scale[a];
                } else if (c >= g->gs[a]) {
                    c -= g->gs[a];
                    sh = g->scale[a];
                }
                if (c < 0 || c >= g->gs[a]) {
                    ok = 0;
                }
            }
            it->c[a] = c;
            it->sh[a] = sh;
        }
        if (!ok) {
            continue;
        }
        if (!g->periodic) {
            const uint32_t rk = (uint32_t)(it->c[0] + g->gs[0] * (it->c[1] + g->gs[1] * it->c[2]));
            if (rk == it->ex0 || rk == it->ex1) {
                continue;
            }
        }
        it->q = 0;
        return 1;
    }
}

static int it_next(orc_iter* it, uint32_t* b, uint32_t* e, float sh[3])
{
    const orc_grid* g = it->g;
    if (it->empty) {
        return 0;
    }
    for (;;) {
        if (it->q >= 8 && !it_next_ref(it)) {
            return 0;
        }
        const int q = it->q++;
        it->t = (uint32_t)((((it->r[2] - it->lo[2]) * (it->hi[1] - it->lo[1] + 1) + (it->r[1] - it->lo[1])) *
                                (it->hi[0] - it->lo[0] + 1) +
                            (it->r[0] - it->lo[0])) *
                               8 +
                           q);
        const int32_t sx = 2 * it->c[0] + (q & 1), sy = 2 * it->c[1] + ((q >> 1) & 1), sz = 2 * it->c[2] + (q >> 2);
        const uint32_t lin = (uint32_t)(sx + g->sgs[0] * (sy + g->sgs[1] * sz));
        if (it->start[lin] == ORC_EMPTY) {
            continue;
        }
        sh[0] = it->sh[0];
        sh[1] = it->sh[1];
        sh[2] = it->sh[2];
        *b = it->start[lin];
        *e = it->end[lin];
        return 1;
    }
}

/* ------------------------------------------------------------------ sort, cells, quirk */
/* Stable LSD radix sort, 8-bit digits (thrust::sort_by_key on int keys is a stable radix sort,
 * cuda/src/simulation/neighbors/NeighborGrid.cu:139-145). */
void orc_sort_stable(uint32_t n, const uint32_t* key, uint32_t bits, uint32_t* perm)
{
    uint32_t* tmp = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    for (uint32_t i = 0; i < n; i++) {
        perm[i] = i;
    }
    for (uint32_t shift = 0; shift < bits; shift += 8) {
        uint32_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (uint32_t i = 0; i < n; i++) {
            cnt[((key[perm[i]] >> shift) & 0xffu) + 1]++;
        }
        for (int d = 0; d < 256; d++) {
            cnt[d + 1] += cnt[d];
        }
        for (uint32_t i = 0; i < n; i++) {
            tmp[cnt[(key[perm[i]] >> shift) & 0xffu]++] = perm[i];
        }
        memcpy(perm, tmp, sizeof(uint32_t) * n);
    }
    free(tmp);
}

/* calculateCellStartAndEndIndices (cuda/src/algorithm/neighbors/NeighborKernels.cu:17-44): thread 0 returns
 * before comparing key[0] with key[1], so when the first two particles of the reference's sorted order lie in
 * different cells, neither cell gets a valid [start, end] and both are skipped by every neighbour query; with
 * one particle its cell is skipped. The reference sorts (cell, array slot); slot order is id order here. */
void orc_excluded_cells(uint32_t n, const uint32_t* refkey, const uint32_t* slot, uint32_t ex[2])
{
    ex[0] = ORC_NONE;
    ex[1] = ORC_NONE;
    if (n == 0) {
        return;
    }
    uint64_t S = ~0ull, T = ~0ull;
    for (uint32_t i = 0; i < n; i++) {
        const uint64_t v = ((uint64_t)refkey[i] << 32) | slot[i];
        if (v < S) {
            T = S;
            S = v;
        } else if (v < T) {
            T = v;
        }
    }
    if (n == 1) {
        ex[0] = (uint32_t)(S >> 32);
        return;
    }
    if ((S >> 32) != (T >> 32)) {
        ex[0] = (uint32_t)(S >> 32);
        ex[1] = (uint32_t)(T >> 32);
    }
}

void orc_cells_from_keys(const orc_grid* g, uint32_t n, const uint32_t* keys, uint32_t* start, uint32_t* end)
{
    for (uint32_t c = 0; c < g->ncells; c++) {
        start[c] = ORC_EMPTY;
        end[c] = 0;
    }
    for (uint32_t k = 0; k < n; k++) {
        const uint32_t lin = lin_of_key(g, keys[k]);
        if (k == 0 || keys[k] != keys[k - 1]) {
            start[lin] = k;
        }
        if (k + 1 == n || keys[k] != keys[k + 1]) {
            end[lin] = k + 1;
        }
    }
}

static void permute_f(float* a, const uint32_t* perm, uint32_t n, int width, float* tmp)
{
    for (uint32_t k = 0; k < n; k++) {
        memcpy(tmp + (size_t)width * k, a + (size_t)width * perm[k], sizeof(float) * width);
    }
    memcpy(a, tmp, sizeof(float) * width * n);
}

void orc_grid_build(const orc_grid* g, orc_state* s, orc_cells* c)
{
    const uint32_t n = s->n;
    const size_t nn = n ? n : 1;
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* refk = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    float* tmp = (float*)malloc(sizeof(float) * 4 * nn);
    for (uint32_t i = 0; i < n; i++) {
        orc_cell_of(g, s->pos + 4 * (size_t)i, &keys[i], &refk[i], NULL);
    }
    if (!g->periodic) {
        orc_excluded_cells(n, refk, s->id, c->ex);
    } else {
        c->ex[0] = c->ex[1] = ORC_NONE;
    }
    orc_sort_stable(n, keys, 3 * g->bits, perm);
    permute_f(s->pos, perm, n, 4, tmp);
    permute_f(s->vel, perm, n, 4, tmp);
    permute_f(s->acc, perm, n, 4, tmp);
    permute_f(s->rho, perm, n, 1, tmp);
    permute_f(s->rad, perm, n, 1, tmp);
    permute_f(s->h, perm, n, 1, tmp);
    permute_f(s->m, perm, n, 1, tmp);
    {
        uint32_t* t = (uint32_t*)tmp;
        for (uint32_t k = 0; k < n; k++) {
            t[k] = s->id[perm[k]];
        }
        memcpy(s->id, t, sizeof(uint32_t) * n);
    }
    for (uint32_t k = 0; k < n; k++) {
        c->keys[k] = keys[perm[k]];
    }
    orc_cells_from_keys(g, n, c->keys, c->start, c->end);
    free(keys);
    free(refk);
    free(perm);
    free(tmp);
}

void orc_boundary_setup(const orc_grid* g, uint32_t n, const float* pos4, const float* psi, float friction,
                        orc_boundary* b)
{
    const size_t nn = n ? n : 1;
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* refk = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* slot = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    for (uint32_t i = 0; i < n; i++) {
        orc_cell_of(g, pos4 + 4 * (size_t)i, &keys[i], &refk[i], NULL);
        slot[i] = i;
    }
    if (!g->periodic) {
        orc_excluded_cells(n, refk, slot, b->ex);
    } else {
        b->ex[0] = b->ex[1] = ORC_NONE;
    }
    orc_sort_stable(n, keys, 3 * g->bits, perm);
    for (uint32_t k = 0; k < n; k++) {
        memcpy(b->pos + 4 * (size_t)k, pos4 + 4 * (size_t)perm[k], sizeof(float) * 4);
        b->psi[k] = psi[perm[k]];
        b->fric[k] = friction;
        slot[k] = keys[perm[k]];
    }
    b->n = n;
    orc_cells_from_keys(g, n, slot, b->start, b->end);
    free(keys);
    free(refk);
    free(slot);
    free(perm);
}

/* ------------------------------------------------------------------ cube root */
/* Cube root by Newton-Raphson on y^3 = a in double precision: x = m * 2^e with the exponent split as
 * e = 3k + r, six iterations y <- (2y + a/y^2)/3 from y = 1 on a = m * 2^r in [0.5, 4), then y * 2^k rounded
 * to float. Only basic IEEE operations, so the CUDA kernels and this oracle produce the same bits. */
float orc_cbrtf(float xf)
{
    if (xf == 0.0f || !(xf == xf) || xf == INFINITY || xf == -INFINITY) {
        return xf;
    }
    const int neg = xf < 0.0f;
    double x = neg ? -(double)xf : (double)xf;
    int e;
    double m = frexp(x, &e);
    int k = e >= 0 ? e / 3 : -((-e + 2) / 3);
    int r = e - 3 * k;
    const double a = ldexp(m, r);
    double y = 1.0;
    for (int it = 0; it < 6; it++) {
        y = ((y + y) + a / (y * y)) / 3.0;
    }
    y = ldexp(y, k);
    const float out = (float)y;
    return neg ? -out : out;
}

/* ------------------------------------------------------------------ FP32 / FP64 bodies */
static const float ORC_PI_F = 3.141592653589793f;
#define ORC_LANES 32       /* lanes of the warp that sums a heavy particle */
#define ORC_HEAVY_CELLS 27 /* query boxes of more reference cells than this are heavy */
#define ORC_LIST_ENTRIES 128 /* neighbour-list row length in entries; a particle needing more is summed by cells */
#define ORC_ROW_HEAVY 96     /* a particle with more row entries than this is summed over its row by a warp */

/* Entries of the particle's neighbour-list row: the candidate cells' members are scanned in blocks of up to 32
 * (counted from each sub-cell's first member); a block in which the particle accepts a neighbour
 * (r^2 <= (2 h_j)^2, self included) is one entry. */
static uint32_t list_entries(const orc_grid* g, const orc_state* s, const orc_cells* c, int64_t i)
{
    const float* pi = s->pos + 4 * i;
    const float R = s->h[i] + s->h[i];
    uint32_t entries = 0;
    orc_iter it;
    uint32_t jb, je;
    float sh[3];
    it_init(&it, g, c->start, c->end, c->ex, pi, R);
    while (it_next(&it, &jb, &je, sh)) {
        for (uint32_t c0 = jb; c0 < je; c0 += 32) {
            const uint32_t c1 = je - c0 < 32u ? je : c0 + 32u;
            int any = 0;
            for (uint32_t j = c0; j < c1 && !any; j++) {
                const float* pj = s->pos + 4 * (size_t)j;
                const float dx = (g->periodic ? pj[0] + sh[0] : pj[0]) - pi[0];
                const float dy = (g->periodic ? pj[1] + sh[1] : pj[1]) - pi[1];
                const float dz = (g->periodic ? pj[2] + sh[2] : pj[2]) - pi[2];
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float twoh = s->h[j] + s->h[j];
                any = r2 <= twoh * twoh;
            }
            entries += any;
        }
    }
    return entries;
}

/* how a particle's sums are dealt to the lanes of a warp (see oracle_body.h) */
enum { ORC_DEAL_NONE = 0, ORC_DEAL_SUBCELL = 1, ORC_DEAL_ENTRY = 2 };

static int sum_kind(const orc_grid* g, const orc_state* s, const orc_cells* c, int64_t i)
{
    const float R = s->h[i] + s->h[i];
    if (box_cells(g, s->pos + 4 * i, R) > ORC_HEAVY_CELLS) {
        return ORC_DEAL_SUBCELL;
    }
    const uint32_t n = list_entries(g, s, c, i);
    if (n > ORC_LIST_ENTRIES) {
        return ORC_DEAL_SUBCELL;
    }
    return n > ORC_ROW_HEAVY ? ORC_DEAL_ENTRY : ORC_DEAL_NONE;
}

/* selection records of the top-k sorts: (key, id) orders them, ids being unique */
typedef struct orc_sel {
    uint64_t key;
    uint32_t id, slot;
} orc_sel;

static int cmp_sel(const void* a, const void* b)
{
    const orc_sel* x = (const orc_sel*)a;
    const orc_sel* y = (const orc_sel*)b;
    if (x->key != y->key) {
        return x->key < y->key ? -1 : 1;
    }
    return x->id < y->id ? -1 : (x->id > y->id ? 1 : 0);
}

static uint32_t sortable_f(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

static uint64_t sortable_d(double f)
{
    uint64_t u;
    memcpy(&u, &f, 8);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

static const float ORC_PHI_F = 1.6180339887498949f;
#define ORC_FOUR_THIRDS_PI 4.18879020478639098461685784437267051226289253250014109463325945641042187504827866483737976712282275730953078202
static const float ORC_INVNORM_F = 0.5257311121f;

/* FP32 canonical arithmetic on the FP32 state (the bit-exact checker) */
#define REAL float
#define SREAL float
#define STATE orc_state
#define ITPOS(p, tmp) ((void)(tmp), (p))
#define SUM_KIND(g, s, c, i) sum_kind(g, s, c, i)
#define F(name) name##_f32
#define FMA fmaf
#define SQRT sqrtf
#define CBRT orc_cbrtf
#define PI_R ORC_PI_F
#define SORTABLE(x) ((uint64_t)sortable_f(x))
#define SORTABLE_DESC(x) ((uint64_t)(uint32_t)~sortable_f(x))
#define WCOEF (21.0f / (16.0f * ORC_PI_F))
#define DCOEF (-5.0f * (21.0f / (16.0f * ORC_PI_F)))
#include "oracle_body.h"
#include "refine_body.h"
#undef REAL
#undef F
#undef FMA
#undef SQRT
#undef WCOEF
#undef DCOEF
#undef NBR

/* FP64 arithmetic on the FP32 state (accuracy reference of one stage on the GPU's own inputs) */
#define REAL double
#define F(name) name##_f64
#define FMA fma
#define SQRT sqrt
#define WCOEF (21.0 / (16.0 * 3.14159265358979323846))
#define DCOEF (-5.0 * (21.0 / (16.0 * 3.14159265358979323846)))
#include "oracle_body.h"
#undef NBR
#undef F
#undef SREAL
#undef STATE
#undef ITPOS
#undef SUM_KIND
#undef CBRT
#undef PI_R
#undef SORTABLE
#undef SORTABLE_DESC

/* FP64 arithmetic on the FP64 state: the FP64 step */
static inline const float* itpos_d64(const double* p, float* tmp)
{
    tmp[0] = (float)p[0];
    tmp[1] = (float)p[1];
    tmp[2] = (float)p[2];
    tmp[3] = 0.0f;
    return tmp;
}
#define SREAL double
#define STATE orc_state64
#define ITPOS(p, tmp) itpos_d64((p), (tmp))
#define SUM_KIND(g, s, c, i) ORC_DEAL_NONE
#define F(name) name##_d64
#define CBRT cbrt
#define PI_R 3.14159265358979323846
#define SORTABLE(x) sortable_d(x)
#define SORTABLE_DESC(x) (~sortable_d(x))
#include "oracle_body.h"
#include "refine_body.h"
#undef REAL
#undef SREAL
#undef STATE
#undef ITPOS
#undef SUM_KIND
#undef F
#undef FMA
#undef SQRT
#undef CBRT
#undef PI_R
#undef SORTABLE
#undef SORTABLE_DESC
#undef WCOEF
#undef DCOEF
#undef NBR

void orc32_density(const orc_grid* g, const orc_params* P, const orc_state* s, const orc_cells* c,
                   const orc_boundary* b, float* rho_out)
{
    orc_density_impl_f32(g, P, s, c, b, rho_out);
}

void orc64_density(const orc_grid* g, const orc_params* P, const orc_state* s, const orc_cells* c,
                   const orc_boundary* b, double* rho_out)
{
    orc_density_impl_f64(g, P, s, c, b, rho_out);
}

void orc32_forces(const orc_grid* g, const orc_params* P, const orc_state* s, const orc_cells* c,
                  const orc_boundary* b, float* acc_out)
{
    orc_forces_impl_f32(g, P, s, c, b, s->rho, acc_out, NULL);
}

void orc64_forces(const orc_grid* g, const orc_params* P, const orc_state* s, const orc_cells* c,
                  const orc_boundary* b, double* acc_out, double* scale_out)
{
    orc_forces_impl_f64(g, P, s, c, b, s->rho, acc_out, scale_out);
}

/* sumAllNeighbors per particle (cuda/src/algorithm/Algorithm.cu:234-268) */
void orc_neighbor_counts(const orc_grid* g, const orc_state* s, const orc_cells* c, uint32_t* counts)
{
    const int64_t n = s->n;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++) {
        const float* pi = s->pos + 4 * i;
        const float R = s->h[i] + s->h[i];
        uint32_t cnt = 0;
        orc_iter it;
        uint32_t jb, je;
        float sh[3];
        it_init(&it, g, c->start, c->end, c->ex, pi, R);
        while (it_next(&it, &jb, &je, sh)) {
            for (uint32_t j = jb; j < je; j++) {
                if ((int64_t)j == i) {
                    continue;
                }
                const float* pj = s->pos + 4 * (size_t)j;
                const float dx = (g->periodic ? pj[0] + sh[0] : pj[0]) - pi[0];
                const float dy = (g->periodic ? pj[1] + sh[1] : pj[1]) - pi[1];
                const float dz = (g->periodic ? pj[2] + sh[2] : pj[2]) - pi[2];
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float twoh = s->h[j] + s->h[j];
                if (r2 <= twoh * twoh) {
                    cnt++;
                }
            }
        }
        counts[i] = cnt;
    }
}

/* ------------------------------------------------------------------ integrator */
/* halfKickVelocities (cuda/src/algorithm/Algorithm.cu:270-284) */
static void kick32(float* v, const float* a, float hdt, float maxv)
{
    v[0] = fmaf(a[0], hdt, v[0]);
    v[1] = fmaf(a[1], hdt, v[1]);
    v[2] = fmaf(a[2], hdt, v[2]);
    const float len = sqrtf(fmaf(v[2], v[2], fmaf(v[1], v[1], v[0] * v[0])));
    if (len > maxv) {
        const float sc = maxv / len;
        v[0] = v[0] * sc;
        v[1] = v[1] * sc;
        v[2] = v[2] * sc;
    }
}

/* The closing half-kick of the previous step is applied here, just before the opening half-kick of this
 * step, then the drift and the domain clamp (updatePositions, Algorithm.cu:286-298); the reference runs the
 * same two kicks as separate kernels at the end and the start of consecutive steps. */
void orc32_integrate(orc_state* s, const orc_params* P, float dt)
{
    const float half = dt / 2.0f;
    const int64_t n = s->n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        float* v = s->vel + 4 * i;
        const float* a = s->acc + 4 * i;
        float* x = s->pos + 4 * i;
        if (s->has_pending) {
            kick32(v, a, s->pending_half, P->max_velocity);
        }
        kick32(v, a, half, P->max_velocity);
        v[3] = 0.0f;
        for (int c = 0; c < 3; c++) {
            float xc = fmaf(v[c], dt, x[c]);
            if (!P->periodic) {
                xc = xc < P->dmin[c] ? P->dmin[c] : xc;
                xc = xc > P->dmax[c] ? P->dmax[c] : xc;
            } else {
                const float L = P->dmax[c] - P->dmin[c];
                if (xc < P->dmin[c]) {
                    xc = xc + L;
                } else if (xc >= P->dmax[c]) {
                    xc = xc - L;
                }
            }
            x[c] = xc;
        }
    }
    s->has_pending = 0;
}

void orc32_export_velocities(const orc_params* P, const orc_state* s, float* vel4_out)
{
    for (uint32_t i = 0; i < s->n; i++) {
        float v[4] = {s->vel[4 * i], s->vel[4 * i + 1], s->vel[4 * i + 2], 0.0f};
        if (s->has_pending) {
            kick32(v, s->acc + 4 * (size_t)i, s->pending_half, P->max_velocity);
        }
        memcpy(vel4_out + 4 * (size_t)i, v, sizeof(v));
    }
}

void orc_totals(const orc_params* P, const orc_state* s, double out[6])
{
    double M = 0, px = 0, py = 0, pz = 0, ke = 0;
    for (uint32_t i = 0; i < s->n; i++) {
        float v[4] = {s->vel[4 * i], s->vel[4 * i + 1], s->vel[4 * i + 2], 0.0f};
        if (s->has_pending) {
            kick32(v, s->acc + 4 * (size_t)i, s->pending_half, P->max_velocity);
        }
        const double m = s->m[i];
        M += m;
        px += m * v[0];
        py += m * v[1];
        pz += m * v[2];
        ke += 0.5 * m * ((double)v[0] * v[0] + (double)v[1] * v[1] + (double)v[2] * v[2]);
    }
    out[0] = M;
    out[1] = px;
    out[2] = py;
    out[3] = pz;
    out[4] = ke;
    out[5] = (double)s->n;
}

/* ------------------------------------------------------------------ refinement */
/* One refinement pass: performAdaptiveRefinement (cuda/src/simulation/AdaptiveSphSimulation.cu:102-113), the body
 * in refine_body.h, on the FP32 state in the canonical FP32 arithmetic */
void orc32_refine(const orc_grid* g, const orc_params* P, const orc_refine* R, orc_state* s, orc_cells* c,
                  orc_report* rep)
{
    refine_impl_f32(g, P, R, s, c, rep);
}

int orc32_step(const orc_grid* g, const orc_params* P, const orc_refine* R, orc_state* s, orc_cells* c,
               const orc_boundary* b, float dt, orc_report* rep)
{
    orc32_integrate(s, P, dt);
    orc_grid_build(g, s, c);
    orc32_density(g, P, s, c, b, s->rho);
    orc32_forces(g, P, s, c, b, s->acc);
    int refined = 0;
    if (R != NULL && R->enabled && R->cooldown > 0) {
        const uint32_t f = s->frame;
        if (f == R->initial_cooldown || (f > R->initial_cooldown && f % R->cooldown == 0)) {
            orc32_refine(g, P, R, s, c, rep);
            refined = 1;
        }
    }
    s->pending_half = dt / 2.0f;
    s->has_pending = 1;
    s->frame++;
    return refined;
}

/* ------------------------------------------------------------------ the FP64 step */
/* The same step as orc32_step on an FP64 state in double arithmetic throughout: integrate, grid, density,
 * forces, refinement (SphSimulation.cu:101-120, AdaptiveSphSimulation.cu:59-85). The grid's cell keys are taken
 * from the positions rounded to float (cells are an acceleration structure: any key of a cell containing the
 * particle visits the same candidates up to the clamp at the box edge). */
static void kick64(double* v, const double* a, double hdt, double maxv)
{
    v[0] = fma(a[0], hdt, v[0]);
    v[1] = fma(a[1], hdt, v[1]);
    v[2] = fma(a[2], hdt, v[2]);
    const double len = sqrt(fma(v[2], v[2], fma(v[1], v[1], v[0] * v[0])));
    if (len > maxv) {
        const double sc = maxv / len;
        v[0] = v[0] * sc;
        v[1] = v[1] * sc;
        v[2] = v[2] * sc;
    }
}

void orc64s_integrate(orc_state64* s, const orc_params* P, double dt)
{
    const double half = dt / 2.0;
    const int64_t n = s->n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double* v = s->vel + 4 * i;
        const double* a = s->acc + 4 * i;
        double* x = s->pos + 4 * i;
        if (s->has_pending) {
            kick64(v, a, s->pending_half, P->max_velocity);
        }
        kick64(v, a, half, P->max_velocity);
        v[3] = 0.0;
        for (int c = 0; c < 3; c++) {
            double xc = fma(v[c], dt, x[c]);
            if (!P->periodic) {
                xc = xc < P->dmin[c] ? P->dmin[c] : xc;
                xc = xc > P->dmax[c] ? P->dmax[c] : xc;
            } else {
                const double L = (double)P->dmax[c] - (double)P->dmin[c];
                if (xc < P->dmin[c]) {
                    xc = xc + L;
                } else if (xc >= P->dmax[c]) {
                    xc = xc - L;
                }
            }
            x[c] = xc;
        }
    }
    s->has_pending = 0;
}

static void permute_d(double* a, const uint32_t* perm, uint32_t n, int width, double* tmp)
{
    for (uint32_t k = 0; k < n; k++) {
        memcpy(tmp + (size_t)width * k, a + (size_t)width * perm[k], sizeof(double) * width);
    }
    memcpy(a, tmp, sizeof(double) * width * n);
}

void orc64s_grid_build(const orc_grid* g, orc_state64* s, orc_cells* c)
{
    const uint32_t n = s->n;
    const size_t nn = n ? n : 1;
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* refk = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * nn);
    double* tmp = (double*)malloc(sizeof(double) * 4 * nn);
    for (uint32_t i = 0; i < n; i++) {
        float pf[4];
        orc_cell_of(g, itpos_d64(s->pos + 4 * (size_t)i, pf), &keys[i], &refk[i], NULL);
    }
    if (!g->periodic) {
        orc_excluded_cells(n, refk, s->id, c->ex);
    } else {
        c->ex[0] = c->ex[1] = ORC_NONE;
    }
    orc_sort_stable(n, keys, 3 * g->bits, perm);
    permute_d(s->pos, perm, n, 4, tmp);
    permute_d(s->vel, perm, n, 4, tmp);
    permute_d(s->acc, perm, n, 4, tmp);
    permute_d(s->rho, perm, n, 1, tmp);
    permute_d(s->rad, perm, n, 1, tmp);
    permute_d(s->h, perm, n, 1, tmp);
    permute_d(s->m, perm, n, 1, tmp);
    {
        uint32_t* t = (uint32_t*)tmp;
        for (uint32_t k = 0; k < n; k++) {
            t[k] = s->id[perm[k]];
        }
        memcpy(s->id, t, sizeof(uint32_t) * n);
    }
    for (uint32_t k = 0; k < n; k++) {
        c->keys[k] = keys[perm[k]];
    }
    orc_cells_from_keys(g, n, c->keys, c->start, c->end);
    free(keys);
    free(refk);
    free(perm);
    free(tmp);
}

void orc64s_density(const orc_grid* g, const orc_params* P, const orc_state64* s, const orc_cells* c,
                    const orc_boundary* b, double* rho_out)
{
    orc_density_impl_d64(g, P, s, c, b, rho_out);
}

void orc64s_forces(const orc_grid* g, const orc_params* P, const orc_state64* s, const orc_cells* c,
                   const orc_boundary* b, double* acc_out)
{
    orc_forces_impl_d64(g, P, s, c, b, s->rho, acc_out, NULL);
}

void orc64s_refine(const orc_grid* g, const orc_params* P, const orc_refine* R, orc_state64* s, orc_cells* c,
                   orc_report* rep)
{
    refine_impl_d64(g, P, R, s, c, rep);
}

int orc64s_step(const orc_grid* g, const orc_params* P, const orc_refine* R, orc_state64* s, orc_cells* c,
                const orc_boundary* b, double dt, orc_report* rep)
{
    orc64s_integrate(s, P, dt);
    orc64s_grid_build(g, s, c);
    orc64s_density(g, P, s, c, b, s->rho);
    orc64s_forces(g, P, s, c, b, s->acc);
    int refined = 0;
    if (R != NULL && R->enabled && R->cooldown > 0) {
        const uint32_t f = s->frame;
        if (f == R->initial_cooldown || (f > R->initial_cooldown && f % R->cooldown == 0)) {
            orc64s_refine(g, P, R, s, c, rep);
            refined = 1;
        }
    }
    s->pending_half = dt / 2.0;
    s->has_pending = 1;
    s->frame++;
    return refined;
}

void orc64s_totals(const orc_params* P, const orc_state64* s, double out[6])
{
    double M = 0, px = 0, py = 0, pz = 0, ke = 0;
    for (uint32_t i = 0; i < s->n; i++) {
        double v[4] = {s->vel[4 * i], s->vel[4 * i + 1], s->vel[4 * i + 2], 0.0};
        if (s->has_pending) {
            kick64(v, s->acc + 4 * (size_t)i, s->pending_half, P->max_velocity);
        }
        const double m = s->m[i];
        M += m;
        px += m * v[0];
        py += m * v[1];
        pz += m * v[2];
        ke += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
    out[0] = M;
    out[1] = px;
    out[2] = py;
    out[3] = pz;
    out[4] = ke;
    out[5] = (double)s->n;
}

/* ------------------------------------------------------------------ boundary generation */
/* Reference kernel in its own operation order (WendlandKernel.cuh:39-52), as StaticBoundaryDomain uses it. */
static float ref_wendland(float r, float h)
{
    const float q = r / h;
    if (q > 2.0f) {
        return 0.0f;
    }
    const float h3 = (h * h) * h;
    const float t = 1.0f - 0.5f * q;
    const float t4 = (t * t) * (t * t);
    return ((21.0f / (16.0f * ORC_PI_F)) / h3) * t4 * (2.0f * q + 1.0f);
}

/* generateWallParticles (StaticBoundaryDomain.cu:88-147) and computePsi (:149-174): psi = rho0 / sum_b W over
 * walls with |d|^2 < (2h)^2 (self included). The reference sums in KD-tree order; this sums in index order. */
uint32_t orc_boundary_generate(const float dmin[3], const float dmax[3], float spacing, float rho0, float h,
                               float* pos4, float* psi, uint32_t cap)
{
    float mn[3], mx[3];
    for (int a = 0; a < 3; a++) {
        mn[a] = dmin[a] - 0.05f;
        mx[a] = dmax[a] + 0.05f;
    }
    size_t n = 0, cap_all = 0;
    float* tmp = NULL;
#define ORC_PUSH(X, Y, Z)                                          \
    do {                                                           \
        if (n == cap_all) {                                        \
            cap_all = cap_all ? cap_all * 2 : 4096;                \
            tmp = (float*)realloc(tmp, sizeof(float) * 4 * cap_all); \
        }                                                          \
        tmp[4 * n] = (X);                                          \
        tmp[4 * n + 1] = (Y);                                      \
        tmp[4 * n + 2] = (Z);                                      \
        tmp[4 * n + 3] = 0.0f;                                     \
        n++;                                                       \
    } while (0)
    for (float x = mn[0]; x < mx[0]; x += spacing)
        for (float z = mn[2]; z < mx[2]; z += spacing) ORC_PUSH(x, mn[1], z);
    for (float x = mn[0]; x < mx[0]; x += spacing)
        for (float z = mn[2]; z < mx[2]; z += spacing) ORC_PUSH(x, mx[1], z);
    for (float y = mn[1] + spacing; y < mx[1]; y += spacing)
        for (float z = mn[2]; z < mx[2]; z += spacing) ORC_PUSH(mn[0], y, z);
    for (float y = mn[1] + spacing; y < mx[1]; y += spacing)
        for (float z = mn[2]; z < mx[2]; z += spacing) ORC_PUSH(mx[0], y, z);
    for (float x = mn[0] + spacing; x < mx[0]; x += spacing)
        for (float y = mn[1] + spacing; y < mx[1]; y += spacing) ORC_PUSH(x, y, mn[2]);
    for (float x = mn[0] + spacing; x < mx[0]; x += spacing)
        for (float y = mn[1] + spacing; y < mx[1]; y += spacing) ORC_PUSH(x, y, mx[2]);
#undef ORC_PUSH
    if (pos4 == NULL || psi == NULL || n > cap || n == 0) {
        free(tmp);
        return (uint32_t)n;
    }
    /* exact radius search through a uniform grid of cell 2h */
    const float R = 2.0f * h;
    const float R2 = R * R;
    int gd[3];
    float lo[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = mn[a] - R;
        gd[a] = (int)((mx[a] + R - lo[a]) / R) + 1;
    }
    const size_t ncell = (size_t)gd[0] * gd[1] * gd[2];
    uint32_t* head = (uint32_t*)malloc(sizeof(uint32_t) * (ncell + 1));
    uint32_t* list = (uint32_t*)malloc(sizeof(uint32_t) * n);
    int* cid = (int*)malloc(sizeof(int) * 3 * n);
    memset(head, 0, sizeof(uint32_t) * (ncell + 1));
    for (size_t i = 0; i < n; i++) {
        int cc[3];
        for (int a = 0; a < 3; a++) {
            cc[a] = (int)((tmp[4 * i + a] - lo[a]) / R);
            cid[3 * i + a] = cc[a];
        }
        head[(size_t)cc[0] + gd[0] * ((size_t)cc[1] + gd[1] * (size_t)cc[2]) + 1]++;
    }
    for (size_t c = 0; c < ncell; c++) {
        head[c + 1] += head[c];
    }
    {
        uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * ncell);
        memcpy(fill, head, sizeof(uint32_t) * ncell);
        for (size_t i = 0; i < n; i++) {
            const size_t c = (size_t)cid[3 * i] + gd[0] * ((size_t)cid[3 * i + 1] + gd[1] * (size_t)cid[3 * i + 2]);
            list[fill[c]++] = (uint32_t)i;
        }
        free(fill);
    }
    const int64_t nn = (int64_t)n;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < nn; i++) {
        float sum = 0.0f;
        /* index-ordered sum: walk all 27 cells, collect, then sum in ascending index order */
        uint32_t buf[4096];
        int nb = 0;
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    const int x = cid[3 * i] + dx, y = cid[3 * i + 1] + dy, z = cid[3 * i + 2] + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= gd[0] || y >= gd[1] || z >= gd[2]) {
                        continue;
                    }
                    const size_t c = (size_t)x + gd[0] * ((size_t)y + gd[1] * (size_t)z);
                    for (uint32_t q = head[c]; q < head[c + 1] && nb < 4096; q++) {
                        const uint32_t j = list[q];
                        const float ddx = tmp[4 * i] - tmp[4 * (size_t)j];
                        const float ddy = tmp[4 * i + 1] - tmp[4 * (size_t)j + 1];
                        const float ddz = tmp[4 * i + 2] - tmp[4 * (size_t)j + 2];
                        const float d2 = (ddx * ddx + ddy * ddy) + ddz * ddz;
                        if (d2 < R2) {
                            buf[nb++] = j;
                        }
                    }
                }
        /* insertion sort of the (short) candidate list by index */
        for (int a = 1; a < nb; a++) {
            const uint32_t v = buf[a];
            int b = a - 1;
            while (b >= 0 && buf[b] > v) {
                buf[b + 1] = buf[b];
                b--;
            }
            buf[b + 1] = v;
        }
        for (int a = 0; a < nb; a++) {
            const uint32_t j = buf[a];
            const float ddx = tmp[4 * i] - tmp[4 * (size_t)j];
            const float ddy = tmp[4 * i + 1] - tmp[4 * (size_t)j + 1];
            const float ddz = tmp[4 * i + 2] - tmp[4 * (size_t)j + 2];
            const float d2 = (ddx * ddx + ddy * ddy) + ddz * ddz;
            sum += ref_wendland(sqrtf(d2), h);
        }
        psi[i] = rho0 * (1.0f / sum);
        memcpy(pos4 + 4 * i, tmp + 4 * i, sizeof(float) * 4);
    }
    free(head);
    free(list);
    free(cid);
    free(tmp);
    return (uint32_t)n;
}

/* per-particle neighbour-list row entries (see list_entries); for tests */
void orc_list_entries(const orc_grid* g, const orc_state* s, const orc_cells* c, uint32_t* out)
{
    const int64_t n = s->n;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++) {
        out[i] = list_entries(g, s, c, i);
    }
}

/* kernel values and the split directions, for the known-answer tests */
double orc64_kernel_w(double r, double h)
{
    double invh, wc, dwc;
    kernel_consts_f64(h, &invh, &wc, &dwc);
    return kernel_w_f64(r, invh, wc);
}

double orc64_kernel_dw(double r, double h)
{
    double invh, wc, dwc;
    kernel_consts_f64(h, &invh, &wc, &dwc);
    return kernel_dw_f64(r, invh, dwc);
}

float orc32_kernel_w(float r, float h)
{
    float invh, wc, dwc;
    kernel_consts_f32(h, &invh, &wc, &dwc);
    return kernel_w_f32(r, invh, wc);
}

void orc_icosahedron(float* out36)
{
    float v[12][3];
    icosahedron_f32(v);
    memcpy(out36, v, sizeof(v));
}

/* how each particle's sums are dealt (0 sequential, 1 by sub-cell, 2 by row entry); for tests */
void orc_sum_kinds(const orc_grid* g, const orc_state* s, const orc_cells* c, uint32_t* out)
{
    const int64_t n = s->n;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++) {
        out[i] = (uint32_t)sum_kind(g, s, c, i);
    }
}
