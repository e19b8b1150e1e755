/*
 * asph_oracle.h — CPU restatement of AdaptiveSph's per-step particle pipeline.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py call it. The product (adaptivesph_gb300) never links, loads or calls it.
 *
 * Parity status: the reference (a-soltysik/AdaptiveSph) ships no tests, golden vectors or fixtures for
 * this path, and its CUDA library cannot be built here (it needs glm 1.0.1 and nanoflann 1.8.0, neither
 * present). Parity with the reference's own outputs is therefore UNPINNED; this restatement is pinned by
 * analytic known answers instead (kernel normalisation, lattice density, icosahedron geometry,
 * split/merge bookkeeping; tests/test_oracle_known_answers.py).
 *
 * Two precisions are compiled from one body (oracle_body.h):
 *   orc32_*  FP32, operation for operation the canonical arithmetic the CUDA kernels use (explicit
 *            fmaf, IEEE division and square root, no contraction), so integer decisions and floats
 *            can be compared bit for bit;
 *   orc64_*  FP64 restatement of the same formulas, the accuracy reference.
 * The canonical arithmetic follows the reference's formulas; the few places where its operation order
 * differs from the reference's are listed beside each function.
 */
#ifndef ASPH_ORACLE_H
#define ASPH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_EMPTY 0xffffffffu
#define ORC_NONE 0xffffffffu

typedef struct orc_params {
    float dmin[3], dmax[3], friction;
    float gravity[3];
    float c0, rho0, restitution, alpha, sigma, max_velocity, h0, r0, m0;
    uint32_t threads_per_block;
    uint32_t viscosity_model; /* 0 artificial (reference), 1 Morris */
    float nu;
    uint32_t periodic;
} orc_params;

typedef struct orc_refine {
    uint32_t enabled;
    float min_mass_ratio, max_mass_ratio;
    uint32_t max_particle_count;
    float max_batch_ratio;
    uint32_t initial_cooldown, cooldown, criterion;
    float eps, alpha, center_ratio, vertex_ratio;
    float vel_split, vel_merge, vort_split, vort_merge, curv_split, curv_merge, iface_split, iface_merge;
    float fs_split, fs_merge; /* free-surface criterion (3): neighbour-count deficit thresholds */
} orc_refine;

typedef struct orc_grid {
    int32_t gs[3];    /* reference grid: ceil(scale / 4h0) (NeighborGrid.cu:108-121) */
    float cs[3];      /* reference cell size scale / gs */
    float scale[3];   /* domain max - min */
    float dmin[3], dmax[3];
    int32_t sgs[3];   /* sub-cells: 2 per reference cell per axis */
    uint32_t ncells;  /* sgs.x * sgs.y * sgs.z */
    uint32_t bits;    /* Morton bits per axis */
    uint32_t periodic;
} orc_grid;

typedef struct orc_state {
    uint32_t n, cap;
    float *pos, *vel, *acc; /* 4 * cap */
    float *rho, *rad, *h, *m;
    uint32_t *id;
    uint32_t frame, next_id, has_pending;
    float pending_half;
} orc_state;

typedef struct orc_cells {
    uint32_t *start, *end; /* ncells */
    uint32_t *keys;        /* n: sub-cell Morton key of each particle in the current order */
    uint32_t ex[2];        /* reference cells skipped by the reference's cell-boundary pass */
} orc_cells;

typedef struct orc_boundary {
    uint32_t n;
    float *pos;  /* 4n, cell-sorted */
    float *psi, *fric;
    uint32_t *start, *end; /* ncells */
    uint32_t ex[2];
} orc_boundary;

typedef struct orc_report {
    uint32_t frame, count_before, merge_eligible, merge_pairs, removed, split_candidates, split_budget, splits,
        count_after, capacity_hit;
    /* optional id lists (NULL to skip): removed ids, merge keep ids, split parent ids (in split order) */
    uint32_t *removed_ids, *keep_ids, *split_ids;
} orc_report;

void orc_set_threads(int n);
int orc_get_threads(void);

void orc_grid_make(const orc_params* P, orc_grid* g);
uint32_t orc_morton3(uint32_t x, uint32_t y, uint32_t z);
/* sub-cell key and reference-cell key of one position (NeighborGrid.cuh:166-177) */
void orc_cell_of(const orc_grid* g, const float* p4, uint32_t* key, uint32_t* refkey, uint32_t* lin);
/* stable LSD radix sort of (key, position): perm[k] = source index of the k-th smallest */
void orc_sort_stable(uint32_t n, const uint32_t* key, uint32_t bits, uint32_t* perm);
/* excluded cells of the reference's calculateCellStartAndEndIndices (NeighborKernels.cu:17-44) */
void orc_excluded_cells(uint32_t n, const uint32_t* refkey, const uint32_t* slot, uint32_t ex[2]);
/* keys, stable sort, permutation of all particle arrays, cell tables; cells->keys ends up cell-sorted */
void orc_grid_build(const orc_grid* g, orc_state* s, orc_cells* c);
void orc_cells_from_keys(const orc_grid* g, uint32_t n, const uint32_t* keys, uint32_t* start, uint32_t* end);
/* boundary: sorts `n` particles by sub-cell (stable by input slot), builds tables; out arrays sized n */
void orc_boundary_setup(const orc_grid* g, uint32_t n, const float* pos4, const float* psi, float friction,
                        orc_boundary* b);
/* StaticBoundaryDomain::generate (StaticBoundaryDomain.cu:76-174); returns the particle count; writes at most cap */
uint32_t orc_boundary_generate(const float dmin[3], const float dmax[3], float spacing, float rho0, float h,
                               float* pos4, float* psi, uint32_t cap);

float orc_cbrtf(float x);

/* FP32 canonical stages */
void orc32_integrate(orc_state* s, const orc_params* P, float dt);
void orc32_density(const orc_grid* g, const orc_params* P, const orc_state* s, const orc_cells* c,
                   const orc_boundary* b, float* rho_out);
void orc32_forces(const orc_grid* g, const orc_params* P, const orc_state* s, const orc_cells* c,
                  const orc_boundary* b, float* acc_out);
void orc_neighbor_counts(const orc_grid* g, const orc_state* s, const orc_cells* c, uint32_t* counts);
/* entries of each particle's neighbour-list row (blocks of <= 32 sub-cell members holding an accepted neighbour) */
void orc_list_entries(const orc_grid* g, const orc_state* s, const orc_cells* c, uint32_t* out);
/* how each particle's sums are dealt to a warp's lanes: 0 sequential, 1 by sub-cell (heavy box or overflowed
 * row), 2 by row entry (long row) */
void orc_sum_kinds(const orc_grid* g, const orc_state* s, const orc_cells* c, uint32_t* out);
/* one refinement pass (AdaptiveSphSimulation.cu:102-252); s must be cell-sorted with valid c */
void orc32_refine(const orc_grid* g, const orc_params* P, const orc_refine* R, orc_state* s, orc_cells* c,
                  orc_report* rep);
/* one full step (SphSimulation.cu:101-120 / AdaptiveSphSimulation.cu:59-85); R may be NULL.
 * c must hold arrays for cap particles and ncells cells. rep may be NULL. Returns 1 if refinement ran. */
int orc32_step(const orc_grid* g, const orc_params* P, const orc_refine* R, orc_state* s, orc_cells* c,
               const orc_boundary* b, float dt, orc_report* rep);

/* FP64 restatement: same inputs (FP32 state), double arithmetic. scale_out (may be NULL) receives, per
 * particle, the sum of |pair terms| of the force, the magnitude against which force errors are measured. */
void orc64_density(const orc_grid* g, const orc_params* P, const orc_state* s, const orc_cells* c,
                   const orc_boundary* b, double* rho_out);
void orc64_forces(const orc_grid* g, const orc_params* P, const orc_state* s, const orc_cells* c,
                  const orc_boundary* b, double* acc_out, double* scale_out);

/* The FP64 step: an FP64 state (same layout and order as orc_state, double arrays) advanced in double arithmetic
 * throughout (integrate, grid, density, forces, refinement), the CPU step the FP32 pipeline is measured against. */
typedef struct orc_state64 {
    uint32_t n, cap;
    double *pos, *vel, *acc; /* 4 * cap */
    double *rho, *rad, *h, *m;
    uint32_t* id;
    uint32_t frame, next_id, has_pending;
    double pending_half;
} orc_state64;

void orc64s_integrate(orc_state64* s, const orc_params* P, double dt);
void orc64s_grid_build(const orc_grid* g, orc_state64* s, orc_cells* c);
void orc64s_density(const orc_grid* g, const orc_params* P, const orc_state64* s, const orc_cells* c,
                    const orc_boundary* b, double* rho_out);
void orc64s_forces(const orc_grid* g, const orc_params* P, const orc_state64* s, const orc_cells* c,
                   const orc_boundary* b, double* acc_out);
void orc64s_refine(const orc_grid* g, const orc_params* P, const orc_refine* R, orc_state64* s, orc_cells* c,
                   orc_report* rep);
int orc64s_step(const orc_grid* g, const orc_params* P, const orc_refine* R, orc_state64* s, orc_cells* c,
                const orc_boundary* b, double dt, orc_report* rep);
void orc64s_totals(const orc_params* P, const orc_state64* s, double out[6]);

/* Wendland kernel W(r, h) and dW/dr (WendlandKernel.cuh:39-84) in both precisions; the 12 split directions
 * (AdaptiveAlgorithm.cu:35-48) as 12 xyz triples */
double orc64_kernel_w(double r, double h);
double orc64_kernel_dw(double r, double h);
float orc32_kernel_w(float r, float h);
void orc_icosahedron(float* out36);

/* FP64 totals: mass, momentum[3], kinetic energy (with the pending half-kick applied) */
void orc_totals(const orc_params* P, const orc_state* s, double out[6]);
/* velocities with the pending closing half-kick applied, as exported (vel4_out: 4n) */
void orc32_export_velocities(const orc_params* P, const orc_state* s, float* vel4_out);

#ifdef __cplusplus
}
#endif
#endif
