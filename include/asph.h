/*
 * asph.h — C ABI of the GB300-native AdaptiveSph per-step particle pipeline.
 *
 * Every entry point replaces one call of the reference's C++ simulation interface
 * (the headers under cuda/include/cuda in a-soltysik/AdaptiveSph). The reference interface each one
 * stands in for is cited beside it as path:line. Plain C types only: pointers, sizes,
 * POD structs. Every call returns an asph_status; asph_last_error() gives the message of
 * the last failing call on the calling thread.
 *
 * Threading: an asph_simulation is used by one host thread at a time (the reference is
 * single-threaded, app/App.cpp:191-251). Work is enqueued on the simulation's CUDA stream;
 * asph_simulation_update() returns after the stream is drained, like the reference's
 * update() which ends in cudaDeviceSynchronize (cuda/src/simulation/SphSimulation.cu:119).
 */
#ifndef ASPH_H
#define ASPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ASPH_ABI_VERSION 1u

typedef enum asph_status {
    ASPH_OK = 0,
    ASPH_ERR_INVALID_ARGUMENT = 1,
    ASPH_ERR_CUDA = 2,
    ASPH_ERR_OUT_OF_MEMORY = 3,
    ASPH_ERR_CAPACITY = 4,
    ASPH_ERR_DEVICE_CHECK = 5, /* the device error word is non-zero; see asph_simulation_device_errors */
    ASPH_ERR_UNSUPPORTED = 6,
    ASPH_ERR_NO_DEVICE = 7
} asph_status;

/* Bits of the device error word (asph_simulation_device_errors). The reference checks none of these. */
#define ASPH_DEVERR_SPIN_LIMIT 0x1u     /* a bounded wait (radix-sort look-back) gave up; results of that step are invalid */
#define ASPH_DEVERR_NONFINITE 0x2u      /* a density or acceleration came out NaN/Inf */
#define ASPH_DEVERR_SPLIT_CAPACITY 0x4u /* splits were dropped because the fluid capacity was reached (informational) */
#define ASPH_DEVERR_ID_OVERFLOW 0x8u    /* the 32-bit particle id space is exhausted */
#define ASPH_DEVERR_ROWS 0x10u          /* a particle lay beyond the allocated neighbour rows; that step is invalid */

/* Simulation::Parameters::Domain (cuda/include/cuda/simulation/Simulation.cuh:66-94) */
typedef struct asph_domain {
    float min[3];
    float max[3];
    float friction;
} asph_domain;

#define ASPH_VISCOSITY_ARTIFICIAL 0u /* the reference's Monaghan-type viscosity (cuda/src/algorithm/Algorithm.cu:110-174) */
#define ASPH_VISCOSITY_MORRIS 1u     /* Morris, Fox & Zhu (1997) laminar viscosity; no reference counterpart */

#define ASPH_BOUNDARY_CLAMP 0u    /* the reference's domain clamp (cuda/src/algorithm/Algorithm.cu:286-298) */
#define ASPH_BOUNDARY_PERIODIC 1u /* periodic box; no reference counterpart */

/* Simulation::Parameters (cuda/include/cuda/simulation/Simulation.cuh:64-109), plus three extension fields. */
typedef struct asph_parameters {
    asph_domain domain;
    float gravity[3];
    float speed_of_sound;
    float rest_density;
    float restitution; /* parsed but unused, as in the reference (Simulation.cuh:100) */
    float viscosity_constant;
    float surface_tension_constant;
    float max_velocity;
    float base_smoothing_radius;
    float base_particle_radius;
    float base_particle_mass;
    uint32_t threads_per_block; /* 0 means the reference default of 256; shapes the split budget exactly as the reference's launch does */
    /* extensions (no reference counterpart) */
    uint32_t viscosity_model;  /* ASPH_VISCOSITY_* */
    float kinematic_viscosity; /* Morris nu [m^2/s] */
    uint32_t boundary_mode;    /* ASPH_BOUNDARY_* */
} asph_parameters;

#define ASPH_CRITERION_VELOCITY 0u  /* refinement/criteria/VelocityCriterion.cuh */
#define ASPH_CRITERION_INTERFACE 1u /* refinement/criteria/InterfaceCriterion.cuh */
#define ASPH_CRITERION_VORTICITY 2u /* refinement/criteria/VorticityCriterion.cuh */
/* Free surface (no reference counterpart): neighbour-count deficit d = 1 - N / N_ref, N the particle's neighbours
 * (|x_i - x_j|^2 <= (2 h_j)^2 over the candidate cells of [x - 2h_i, x + 2h_i], self excluded) and
 * N_ref = (4 pi / 3) (2 h_i)^3 rho0 / m_i - 1 the count a uniform medium of its own volume would give. Split where
 * d >= free_surface_split_deficit (score d), except within 2 h_i of a domain face (there the domain clamp, not the
 * air, truncates the support) and where the daughters would leave the domain (as for the other criteria); merge where
 * d <= free_surface_merge_deficit (score (max(d, 0) + t) / 2t, t the merge deficit: deep bulk first). */
#define ASPH_CRITERION_FREE_SURFACE 3u

/* refinement::RefinementParameters with its nested parameter structs
 * (cuda/include/cuda/refinement/RefinementParameters.cuh:6-104), flattened. */
typedef struct asph_refinement_parameters {
    uint32_t enabled;
    float min_mass_ratio;
    float max_mass_ratio;
    uint32_t max_particle_count;
    float max_batch_ratio;
    uint32_t initial_cooldown;
    uint32_t cooldown;
    uint32_t criterion; /* ASPH_CRITERION_* */
    /* SplittingParameters (RefinementParameters.cuh:72-78) */
    float split_epsilon;
    float split_alpha;
    float split_center_mass_ratio;
    float split_vertex_mass_ratio;
    /* VelocityParameters (:8-22) */
    float velocity_split_min_speed;
    float velocity_merge_max_speed;
    /* VorticityParameters (:24-38) */
    float vorticity_split_min;
    float vorticity_merge_max;
    /* CurvatureParameters (:40-54): parsed but unused, as in the reference */
    float curvature_split_min;
    float curvature_merge_max;
    /* InterfaceParameters (:56-70) */
    float interface_split_distance_ratio;
    float interface_merge_distance_ratio;
    /* extension (no reference counterpart): the free-surface criterion's thresholds */
    float free_surface_split_deficit;
    float free_surface_merge_deficit;
} asph_refinement_parameters;

/* Fills *p with the reference's defaults (RefinementParameters.cuh:8-104). */
void asph_refinement_parameters_default(asph_refinement_parameters* p);

/* physics::StaticBoundaryDomain::Particle (cuda/include/cuda/simulation/physics/StaticBoundaryDomain.cuh:17-21) */
typedef struct asph_boundary_particle {
    float position[4];
    float psi;
} asph_boundary_particle;

/* Simulation::DensityInfo (cuda/include/cuda/simulation/Simulation.cuh:111-120) */
typedef struct asph_density_info {
    float rest_density;
    float min_density;
    float max_density;
    float average_density;
    uint32_t under_density_count;
    uint32_t normal_density_count;
    uint32_t over_density_count;
} asph_density_info;

/* FP64 conserved totals over the fluid (no reference counterpart). Velocities include the pending closing half-kick. */
typedef struct asph_totals {
    double mass;
    double momentum[3];
    double kinetic_energy;
    double volume; /* sum of m/rho over particles with rho > 0 */
    uint32_t count;
} asph_totals;

/* ---------------------------------------------------------------------------------------------
 * Imported memory: ImportedMemory / importBuffer (cuda/include/cuda/memory/ImportedMemory.cuh:10-26,
 * implemented by cuda/src/memory/ImportedParticleMemory.cu:36-63).
 * ------------------------------------------------------------------------------------------- */
typedef struct asph_memory asph_memory;

/* importBuffer(int handle, size_t size) (ImportedMemory.cuh:25): imports an opaque POSIX file descriptor
 * exported by Vulkan. Ownership of fd passes to CUDA on success. */
asph_status asph_import_buffer_fd(int fd, size_t size, asph_memory** out);
/* Headless stand-in for a Vulkan-exported buffer: a plain device allocation of `size` bytes. */
asph_status asph_memory_allocate(size_t size, asph_memory** out);
/* ImportedParticleMemory::getData<T>() / getSize() (cuda/src/memory/ImportedParticleMemory.cuh:27-36) */
asph_status asph_memory_device_pointer(const asph_memory* mem, void** out);
asph_status asph_memory_size(const asph_memory* mem, size_t* out);
/* ~ImportedParticleMemory (cuda/src/memory/ImportedParticleMemory.cu:13-17) */
void asph_memory_release(asph_memory* mem);

/* FluidParticlesDataImportedBuffer (Simulation.cuh:46-52): vec4 positions, vec4 velocities, float densities,
 * float radii; each holds at least capacity elements. */
typedef struct asph_fluid_buffers {
    const asph_memory* positions;
    const asph_memory* velocities;
    const asph_memory* densities;
    const asph_memory* radii;
} asph_fluid_buffers;

/* BoundaryParticlesDataImportedBuffer (Simulation.cuh:54-59): vec4 positions, float radii, vec4 colors. */
typedef struct asph_boundary_buffers {
    const asph_memory* positions;
    const asph_memory* radii;
    const asph_memory* colors;
} asph_boundary_buffers;

/* ---------------------------------------------------------------------------------------------
 * Boundary domain: StaticBoundaryDomain::generate (StaticBoundaryDomain.cuh:23-26,
 * cuda/src/simulation/physics/StaticBoundaryDomain.cu:76-174). Host code.
 * With out == NULL only *count is written. Otherwise at most `capacity` particles are written and
 * ASPH_ERR_CAPACITY is returned if more exist.
 * ------------------------------------------------------------------------------------------- */
asph_status asph_boundary_generate(const asph_domain* bounds,
                                   float particle_spacing,
                                   float fluid_rest_density,
                                   float fluid_smoothing_radius,
                                   asph_boundary_particle* out,
                                   uint32_t capacity,
                                   uint32_t* count);

/* StaticBoundaryDomain::generate on the GPU (StaticBoundaryDomain.cu:76-174 runs on the host in the reference):
 * the same contract and bit-identical output as asph_boundary_generate (positions from the reference's float
 * loops, psi summed in the same order); with out == NULL only *count is written (host arithmetic only). */
asph_status asph_boundary_generate_gpu(const asph_domain* bounds,
                                       float particle_spacing,
                                       float fluid_rest_density,
                                       float fluid_smoothing_radius,
                                       asph_boundary_particle* out,
                                       uint32_t capacity,
                                       uint32_t* count);

/* ---------------------------------------------------------------------------------------------
 * Simulation (cuda/include/cuda/simulation/Simulation.cuh:61-145)
 * ------------------------------------------------------------------------------------------- */
typedef struct asph_simulation asph_simulation;

/* createSimulation (Simulation.cuh:138-145, cuda/src/simulation/SimulationFactory.cu:14-40).
 * positions: `count` xyzw float quadruples on the host. fluid_buffers / boundary_buffers may be NULL
 * (headless). refinement may be NULL; when refinement->enabled the fluid capacity is
 * refinement->max_particle_count (cuda/src/simulation/AdaptiveSphSimulation.cu:37), otherwise
 * max_fluid_capacity. */
asph_status asph_simulation_create(const asph_parameters* parameters,
                                   const float* positions,
                                   uint32_t count,
                                   const asph_fluid_buffers* fluid_buffers,
                                   const asph_boundary_buffers* boundary_buffers,
                                   const asph_boundary_particle* boundary,
                                   uint32_t boundary_count,
                                   const asph_refinement_parameters* refinement,
                                   uint32_t max_fluid_capacity,
                                   uint32_t max_boundary_capacity,
                                   asph_simulation** out);

/* StaticBoundaryDomain::generate(domain, wall_spacing, rest_density, base_smoothing_radius) followed by
 * createSimulation (app/App.cpp:144-172), with the walls generated on the device and handed to the simulation without
 * a trip through host memory (no reference counterpart for the device path). The walls equal those of
 * asph_boundary_generate bit for bit, so the simulation equals one created from them. */
asph_status asph_simulation_create_with_walls(const asph_parameters* parameters,
                                              const float* positions,
                                              uint32_t count,
                                              const asph_fluid_buffers* fluid_buffers,
                                              const asph_boundary_buffers* boundary_buffers,
                                              float wall_spacing,
                                              const asph_refinement_parameters* refinement,
                                              uint32_t max_fluid_capacity,
                                              uint32_t max_boundary_capacity,
                                              asph_simulation** out);

/* Simulation::~Simulation */
void asph_simulation_destroy(asph_simulation* sim);

/* Simulation::update(float deltaTime) (Simulation.cuh:124; SphSimulation.cu:101-120,
 * AdaptiveSphSimulation.cu:59-85). Enqueues one step and drains the stream. */
asph_status asph_simulation_update(asph_simulation* sim, float delta_time);

/* Enqueues one step without draining the stream (no reference counterpart). Steps that contain a
 * refinement pass still read the new particle count back once. */
asph_status asph_simulation_step_async(asph_simulation* sim, float delta_time);

/* One step with dt = cfl * min_i h_i / (c0 + |v_i|), capped at dt_max when dt_max > 0; the dt used is
 * written to *dt_used (no reference counterpart: the reference takes dt from its caller, app/App.cpp:230). */
asph_status asph_simulation_step_cfl(asph_simulation* sim, float cfl, float dt_max, float* dt_used);

/* Drains the simulation's stream (and the copies of an asynchronous export) and checks the device error word. */
asph_status asph_simulation_synchronize(asph_simulation* sim);

/* Simulation::updateDomain (Simulation.cuh:125-126; SphSimulation.cu:122-134). */
asph_status asph_simulation_update_domain(asph_simulation* sim,
                                          const asph_domain* domain,
                                          const asph_boundary_particle* boundary,
                                          uint32_t boundary_count);

/* getFluidParticlesCount / getBoundaryParticlesCount (Simulation.cuh:128-129) */
asph_status asph_simulation_fluid_count(const asph_simulation* sim, uint32_t* out);
asph_status asph_simulation_boundary_count(const asph_simulation* sim, uint32_t* out);

/* calculateAverageNeighborCount (Simulation.cuh:131; SphSimulation.cu:237-247) */
asph_status asph_simulation_average_neighbor_count(asph_simulation* sim, float* out);

/* getDensityInfo(float threshold) (Simulation.cuh:133; SphSimulation.cu:249-285) */
asph_status asph_simulation_density_info(asph_simulation* sim, float threshold, asph_density_info* out);

/* enableAdaptiveRefinement (Simulation.cuh:135; cuda/src/simulation/AdaptiveSphSimulation.cu:87-90; no-op when plain,
 * SphSimulation.cu:365) */
asph_status asph_simulation_enable_adaptive_refinement(asph_simulation* sim);

/* Writes positions, velocities, densities and radii of [0, count) into the imported fluid buffers (the
 * reference writes them in place every step; here the export is explicit because the internal state is
 * kept cell-sorted). Velocities include the pending closing half-kick. Drains the stream. */
asph_status asph_simulation_export(asph_simulation* sim);

/* Copies the export arrays to host memory instead (pinned or pageable). Any pointer may be NULL.
 * positions/velocities: 4*count floats; densities/radii: count floats; ids: count uint32. */
asph_status asph_simulation_export_host(asph_simulation* sim,
                                        float* positions,
                                        float* velocities,
                                        float* densities,
                                        float* radii,
                                        uint32_t* ids,
                                        uint32_t capacity);

/* The same export without waiting (no reference counterpart): the export kernel is enqueued behind the steps
 * already enqueued and the device-to-host copies run on a copy stream of the simulation, so later steps overlap
 * them. The host arrays (pinned for the copies to be asynchronous) must stay valid and must not be read until
 * asph_simulation_export_wait returns. At most one such export is in flight: the next one reuses the staging
 * buffer after the previous copies (a device-side wait, not a host one). */
asph_status asph_simulation_export_host_async(asph_simulation* sim,
                                              float* positions,
                                              float* velocities,
                                              float* densities,
                                              float* radii,
                                              uint32_t* ids,
                                              uint32_t capacity);
/* Waits for the copies of the last asph_simulation_export_host_async and checks the device error word. */
asph_status asph_simulation_export_wait(asph_simulation* sim);

/* FP64 totals (no reference counterpart). */
asph_status asph_simulation_totals(asph_simulation* sim, asph_totals* out);

/* Device error word, ASPH_DEVERR_* bits, accumulated since create; `clear` resets it. */
asph_status asph_simulation_device_errors(asph_simulation* sim, uint32_t* out, int clear);

/* Uses the given cudaStream_t (as void*) for all further work; NULL selects the simulation's own stream. */
asph_status asph_simulation_set_stream(asph_simulation* sim, void* cuda_stream);

/* ---------------------------------------------------------------------------------------------
 * State access for checkpoints and parity tests (no reference counterpart). Arrays are in the
 * simulation's internal order (cell-sorted after each step, newly split particles appended).
 * positions, velocities, accelerations: 4*count floats (w of velocity/acceleration is 0);
 * densities, radii, smoothing_radii, masses: count floats; ids: count uint32 (a particle's id orders it
 * like the reference's array slot). Any pointer may be NULL on read.
 * ------------------------------------------------------------------------------------------- */
typedef struct asph_state_info {
    uint32_t count;
    uint32_t capacity;
    uint32_t frame;        /* the reference's _frameCounter (cuda/src/simulation/AdaptiveSphSimulation.cuh:43) */
    uint32_t next_id;      /* id given to the next new particle */
    float pending_half_dt; /* closing half-kick not yet applied to the stored velocities */
    uint32_t has_pending;
} asph_state_info;

asph_status asph_simulation_state_info(asph_simulation* sim, asph_state_info* out);
asph_status asph_simulation_read_fluid(asph_simulation* sim,
                                       float* positions,
                                       float* velocities,
                                       float* accelerations,
                                       float* densities,
                                       float* radii,
                                       float* smoothing_radii,
                                       float* masses,
                                       uint32_t* ids,
                                       uint32_t capacity);
/* Replaces the whole fluid state; all pointers are required. */
asph_status asph_simulation_write_fluid(asph_simulation* sim,
                                        const asph_state_info* info,
                                        const float* positions,
                                        const float* velocities,
                                        const float* accelerations,
                                        const float* densities,
                                        const float* radii,
                                        const float* smoothing_radii,
                                        const float* masses,
                                        const uint32_t* ids);

/* Runs the stages of one step up to and including `last_stage`, then stops (for kernel-level parity
 * tests). A full step is ASPH_STAGE_ALL. After ASPH_STAGE_FORCES the step is finished except for the
 * refinement pass and the frame/pending-kick bookkeeping. */
#define ASPH_STAGE_INTEGRATE 1u
#define ASPH_STAGE_GRID 2u
#define ASPH_STAGE_DENSITY 3u
#define ASPH_STAGE_FORCES 4u
#define ASPH_STAGE_ALL 5u
asph_status asph_simulation_run_stages(asph_simulation* sim, float delta_time, uint32_t last_stage);

/* Cell-sorted keys and cell tables of the fluid grid built by the last GRID stage. keys: count uint32 Morton
 * keys of the sub-cells in internal order; cell_start/cell_end: cell_count uint32 each (start == 0xffffffff
 * for an empty cell); excluded_cells: the two reference grid cells skipped by the reference's
 * cell-boundary pass (0xffffffff when none). */
typedef struct asph_grid_info {
    int32_t reference_cells[3];
    float reference_cell_size[3];
    int32_t sub_cells[3];
    uint32_t cell_count;
    uint32_t key_bits;
    uint32_t excluded_cells[2];
    uint32_t boundary_excluded_cells[2];
} asph_grid_info;
asph_status asph_simulation_grid_info(asph_simulation* sim, asph_grid_info* out);
asph_status asph_simulation_read_grid(asph_simulation* sim,
                                      uint32_t* keys,
                                      uint32_t key_capacity,
                                      uint32_t* cell_start,
                                      uint32_t* cell_end,
                                      uint32_t cell_capacity);

/* Per-particle neighbour counts #{j != i : |x_i-x_j|^2 <= (2h_j)^2} over the reference's candidate cells
 * (the per-particle terms of sumAllNeighbors, cuda/src/algorithm/Algorithm.cu:234-268). */
asph_status asph_simulation_neighbor_counts(asph_simulation* sim, uint32_t* counts, uint32_t capacity);

/* Statistics of the last refinement pass. */
typedef struct asph_refinement_report {
    uint32_t frame;
    uint32_t count_before;
    uint32_t merge_eligible;   /* eligibleCount (AdaptiveAlgorithm.cuh:96-131) */
    uint32_t merge_pairs;      /* mergeCount (AdaptiveAlgorithm.cu:208-234) */
    uint32_t removed;          /* particles removed by compaction */
    uint32_t split_candidates; /* particlesSplitCount on the device (AdaptiveAlgorithm.cuh:56-94) */
    uint32_t split_budget;     /* min(candidates, removed/12) (AdaptiveSphSimulation.cu:178-179) */
    uint32_t splits;           /* parents actually split */
    uint32_t count_after;
} asph_refinement_report;
asph_status asph_simulation_last_refinement(asph_simulation* sim, asph_refinement_report* out);

/* Per-kernel device time, recorded with CUDA events on the launching stream while enabled. */
#define ASPH_KERNEL_INTEGRATE 0u
#define ASPH_KERNEL_SORT 1u
#define ASPH_KERNEL_REORDER 2u
#define ASPH_KERNEL_DENSITY 3u
#define ASPH_KERNEL_FORCES 4u
#define ASPH_KERNEL_REFINE 5u
/* the phases of a refinement pass (each also inside ASPH_KERNEL_REFINE): merge scores and their selection sorts;
 * candidates, pairing and merges; compaction; split scores and their selection sorts; splits and the read-back */
#define ASPH_KERNEL_REFINE_MERGE_SELECT 6u
#define ASPH_KERNEL_REFINE_MERGE 7u
#define ASPH_KERNEL_REFINE_COMPACT 8u
#define ASPH_KERNEL_REFINE_SPLIT_SELECT 9u
#define ASPH_KERNEL_REFINE_SPLIT 10u
#define ASPH_KERNEL_COUNT 11u
asph_status asph_simulation_enable_timing(asph_simulation* sim, int enable);
/* ms[k]: summed event time of kernel class k since enabling; launches[k]: launches timed. Drains the stream. */
asph_status asph_simulation_kernel_times(asph_simulation* sim, double* ms, uint32_t* launches, uint32_t n);
/* Number of kernels this library launched on the simulation's stream since create (all classes). */
asph_status asph_simulation_launch_count(const asph_simulation* sim, uint64_t* out);

/* Device memory a simulation can hold, and the same figure for a simulation not yet created; no reference
 * counterpart. Both are the figure at the fluid capacity: the neighbour rows (1 KB per particle) are allocated for
 * the particles present plus headroom and grown, up to the capacity, by the step that needs more. */
asph_status asph_simulation_device_bytes(const asph_simulation* sim, uint64_t* out);
asph_status asph_estimate_device_bytes(const asph_parameters* parameters,
                                       uint32_t count,
                                       uint32_t boundary_count,
                                       const asph_refinement_parameters* refinement,
                                       uint32_t max_fluid_capacity,
                                       uint32_t max_boundary_capacity,
                                       uint64_t* out);

/* ---------------------------------------------------------------------------------------------
 * Batches (no reference counterpart): independent simulations advanced together. Each simulation
 * keeps its own streams, so their steps overlap on the device; plain steps are captured once as
 * CUDA graphs and replayed. A batch does not own its simulations; while a batch step runs, the
 * simulations must not be used otherwise. Every simulation's result equals the one it gives when
 * stepped alone.
 * ------------------------------------------------------------------------------------------- */
typedef struct asph_batch asph_batch;
/* sims[count]: distinct simulations, each on its own stream (the default: set_stream not called with
 * the legacy default stream). */
asph_status asph_batch_create(asph_simulation* const* sims, uint32_t count, asph_batch** out);
void asph_batch_destroy(asph_batch* batch);
/* Advances simulation k by `steps` steps of dts[k]; returns when all of them have finished, after
 * checking every simulation's device error word. */
asph_status asph_batch_step(asph_batch* batch, const float* dts, uint32_t steps);
/* Steps replayed from graphs, steps run eagerly (refinement frames), graph captures so far. */
asph_status asph_batch_stats(const asph_batch* batch, uint64_t* graph_steps, uint64_t* eager_steps,
                             uint64_t* captures);
/* How plain frames are stepped. GRAPHS: one captured graph per simulation step, the simulations' graphs
 * overlapping on their own streams. SEGMENTED: every plain-stepping simulation's grid stage on its own stream, then
 * its density and force passes inside segmented launches shared by up to 64 simulations (persistent kernels walking
 * a queue of 128-particle work items), the whole batch step one captured graph. AUTO (the default): an autotuner
 * times the choices over the batch's first plain frames (per particle-count bucket -- below 16k, below 64k, above --
 * segmented or per-simulation graphs; work items per CTA turn; persistent CTAs per SM) and keeps the fastest.
 * Every mode gives every simulation the same result bit for bit. */
#define ASPH_BATCH_AUTO 0u
#define ASPH_BATCH_GRAPHS 1u
#define ASPH_BATCH_SEGMENTED 2u
asph_status asph_batch_set_mode(asph_batch* batch, uint32_t mode);
#define ASPH_BATCH_MAX_TRIALS 16u
typedef struct asph_batch_tuning_info {
    uint32_t mode;
    uint32_t tuned;           /* 1 once the autotuner has chosen */
    uint32_t segmented[3];    /* per bucket: 1 segmented, 0 per-simulation graphs */
    uint32_t chunk;           /* consecutive work items per CTA turn */
    uint32_t ctas_per_sm;     /* CTAs per SM of the ordinary segmented kernels (persistent); 0: one CTA per turn */
    uint32_t trials;          /* configurations timed */
    uint64_t segmented_steps; /* batch steps run through the segmented graph */
    uint64_t segmented_captures;
    double trial_ms[ASPH_BATCH_MAX_TRIALS];        /* wall time of one plain frame of the whole batch */
    uint32_t trial_config[ASPH_BATCH_MAX_TRIALS];  /* bits 0-2 segmented per bucket, 8-15 chunk, 16-23 CTAs/SM */
} asph_batch_tuning_info;
asph_status asph_batch_tuning(const asph_batch* batch, asph_batch_tuning_info* out);

/* ---------------------------------------------------------------------------------------------
 * Serving loop (no reference counterpart): scene requests are submitted at any time, admitted first
 * come first served while the device memory they need (asph_estimate_device_bytes, capacity
 * included, so split headroom is reserved at admission) fits the budget, advanced together with all
 * other admitted requests (their steps overlap on the device, as in a batch), and retired when their
 * step count is reached: the particles are copied to host memory and the device memory returns to
 * the budget. Each request's result equals the one it gives when run alone. Times are seconds since
 * the server's creation (monotonic clock).
 * ------------------------------------------------------------------------------------------- */
typedef struct asph_server asph_server;

typedef struct asph_request {
    asph_parameters parameters;
    const float* positions; /* host, 4 floats per particle; copied at submission */
    uint32_t count;
    const asph_boundary_particle* boundary; /* host; copied at submission */
    uint32_t boundary_count;
    const asph_refinement_parameters* refinement; /* NULL or disabled: plain */
    uint32_t max_fluid_capacity;                  /* plain: at least count (adaptive: refinement->max_particle_count) */
    float delta_time;
    uint32_t steps;
    /* > 0 with boundary_count == 0: walls of this spacing are generated on the GPU at admission
     * (asph_simulation_create_with_walls) instead of being passed in */
    float wall_spacing;
} asph_request;

#define ASPH_REQUEST_QUEUED 0u
#define ASPH_REQUEST_ACTIVE 1u
#define ASPH_REQUEST_DONE 2u
#define ASPH_REQUEST_FAILED 3u

typedef struct asph_request_status {
    uint32_t state; /* ASPH_REQUEST_* */
    uint32_t steps_done;
    uint32_t steps;
    uint32_t count;      /* particles of the result (done) */
    asph_status error;   /* failed: why */
    uint64_t device_bytes;
    double submit_s, admit_s, finish_s;
} asph_request_status;

/* max_active: most requests running at once (0: 1024). */
asph_status asph_server_create(uint64_t memory_budget_bytes, uint32_t max_active, asph_server** out);
/* Releases every request, finished or not. */
void asph_server_destroy(asph_server* server);
/* Queues a request; ASPH_ERR_CAPACITY if it could never fit the budget. May be called from another
 * thread than the one polling. */
asph_status asph_server_submit(asph_server* server, const asph_request* request, uint64_t* ticket);
/* Admits what fits, advances every running request by up to max_steps steps (0: to its end), retires
 * the finished ones; returns when those steps are done. *outstanding: requests queued or running. */
asph_status asph_server_poll(asph_server* server, uint32_t max_steps, uint32_t* outstanding);
asph_status asph_server_status(asph_server* server, uint64_t ticket, asph_request_status* out);
/* Copies a finished request's particles (as asph_simulation_export_host) and forgets the request; a
 * failed request returns its error and is forgotten. */
asph_status asph_server_take(asph_server* server, uint64_t ticket, float* positions, float* velocities,
                             float* densities, float* radii, uint32_t* ids, uint32_t capacity);
asph_status asph_server_stats(const asph_server* server, uint64_t* used_bytes, uint32_t* queued, uint32_t* active,
                              uint64_t* graph_steps, uint64_t* eager_steps);

/* ---------------------------------------------------------------------------------------------
 * Cell sort without allocation. No counterpart in the reference: it is the cell-key computation and
 * stable key sort of NeighborGrid::update (cuda/src/simulation/neighbors/NeighborGrid.cu:123-150)
 * plus the cell tables, offered alone for callers that must not allocate device memory. Such
 * callers own all device memory through their own allocator (a renderer that imports its particle
 * buffers into CUDA under a fixed budget) or run in a frame loop where cudaMalloc/cudaFree would
 * stall other streams (cudaFree synchronises the device) or could fail mid-frame.
 *
 * The call allocates nothing: its scratch is one fixed array of device memory inside this library
 * (about 4.9 MB, sized for ASPH_NOALLOC_MAX_PARTICLES). count > ASPH_NOALLOC_MAX_PARTICLES is
 * rejected with ASPH_ERR_CAPACITY. Every call made outside stream capture looks up the scratch
 * address on the current device (the first one, with lazy module loading, also loads the library's
 * device code there), so a device reset between calls is followed; a captured call reuses the address
 * of the last uncaptured call on that device, so make the first call on each device before any stream
 * capture (a first call inside a capture is refused). The scratch is shared by all calls on a device: calls
 * that may overlap (different streams, or several host threads) race on it and must be serialised
 * by the caller. The sort's counters are zeroed by the call itself on `stream`; nothing in the
 * scratch has to start at zero. The caller zeroes `device_errors` before its first use.
 *
 * params:        grid as asph_simulation_create builds it (domain, base_smoothing_radius, boundary_mode)
 * positions:     device, 4 floats per particle (x, y, z, unused)
 * sorted_keys:   device [count], sub-cell keys in sorted order (bit-identical to asph_simulation_read_grid)
 * order:         device [count], order[k] = input index of the k-th particle (stable: equal keys keep
 *                their input order)
 * cell_start, cell_end: device [asph_grid_info.cell_count] or both NULL; cell_capacity their length
 * device_errors: device word, OR-ed with ASPH_DEVERR_SPIN_LIMIT if a bounded wait of the sort gave up
 * stream:        cudaStream_t (NULL: the legacy default stream); the call is asynchronous on it.
 * ------------------------------------------------------------------------------------------- */
#define ASPH_NOALLOC_MAX_PARTICLES 524288u
asph_status asph_grid_sort_noalloc(const asph_parameters* params,
                                   const float* positions,
                                   uint32_t count,
                                   uint32_t* sorted_keys,
                                   uint32_t* order,
                                   uint32_t* cell_start,
                                   uint32_t* cell_end,
                                   uint32_t cell_capacity,
                                   uint32_t* device_errors,
                                   void* stream);

/* ---------------------------------------------------------------------------------------------
 * Misc
 * ------------------------------------------------------------------------------------------- */
uint32_t asph_abi_version(void);
const char* asph_status_string(asph_status status);
const char* asph_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* ASPH_H */
