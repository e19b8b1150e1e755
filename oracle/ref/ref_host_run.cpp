// ref_host_run.cpp — runs AdaptiveSph's own CUDA kernels on the CPU, as a checker of the oracle and of the CUDA
// pipeline (TEST INFRASTRUCTURE ONLY: built into oracle/_ref/ by oracle/ref/build.py from the reference's sources
// where they lie; never part of the product, never shipped).
//
// The reference's kernel translation units (cuda/src/algorithm/Algorithm.cu, BoundaryAlgorithm.cu,
// AdaptiveAlgorithm.cu, algorithm/neighbors/NeighborKernels.cu) and its boundary generator
// (cuda/src/simulation/physics/StaticBoundaryDomain.cu) are compiled unchanged as host C++ (g++, Thrust on its CPP
// system). This file supplies what nvcc and the CUDA runtime would: a launcher that runs a kernel's threads in turn
// (blocks spread over OpenMP threads where the kernel's threads are independent, strictly in order where the kernel
// orders its work through atomics), host-memory stand-ins for the few runtime calls of the reference's headers, and
// the host orchestration of the reference's classes, restated from their sources because those files also hold
// kernel launches (<<<...>>>), which only nvcc parses:
//   SphSimulation::update ................ cuda/src/simulation/SphSimulation.cu:101-120
//   AdaptiveSphSimulation::update ........ cuda/src/simulation/AdaptiveSphSimulation.cu:59-85
//   performAdaptiveRefinement ............ AdaptiveSphSimulation.cu:102-113
//   resetRefinementCounters .............. AdaptiveSphSimulation.cu:115-133
//   identifyAndSplitParticles ............ AdaptiveSphSimulation.cu:135-193
//   identifyAndMergeParticles ............ AdaptiveSphSimulation.cu:195-252
//   calculateMergeCriteria ............... AdaptiveSphSimulation.cu:254-285
//   NeighborGrid (grid size, update) ..... cuda/src/simulation/neighbors/NeighborGrid.cu:33-150
//   SphSimulation constructor state ...... SphSimulation.cu:28-80 (velocities 0, accelerations = gravity, h0, m0, r0)
//   calculateAverageNeighborCount ........ SphSimulation.cu:237-247
//   getDensityInfo ....................... SphSimulation.cu:249-285
// The reference keeps no particle ids; the checker carries one per particle through the same moves (stable
// compaction, daughters appended in split-thread order) so that results can be matched to the oracle's particles.
#include <omp.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <optional>
#include <vector>

#include "algorithm/AdaptiveAlgorithm.cuh"
#include "algorithm/Algorithm.cuh"
#include "algorithm/BoundaryAlgorithm.cuh"
#include "algorithm/WendlandKernel.cuh"
#include "algorithm/neighbors/NeighborKernels.cuh"
#include "asph_oracle.h"
#include "cuda/simulation/physics/StaticBoundaryDomain.cuh"
#include "simulation/refinement/Common.cuh"
#include "simulation/refinement/criteria/InterfaceCriterion.cuh"
#include "simulation/refinement/criteria/VelocityCriterion.cuh"
#include "simulation/refinement/criteria/VorticityCriterion.cuh"

thread_local asph_ref_host::Coord threadIdx{0, 0, 0};
thread_local asph_ref_host::Coord blockIdx{0, 0, 0};
thread_local asph_ref_host::Coord blockDim{1, 1, 1};
thread_local asph_ref_host::Coord gridDim{1, 1, 1};

// ------------------------------------------------------------------ CUDA runtime stand-ins (host memory)
extern "C" {
cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::calloc(n ? n : 1, 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    std::memmove(d, s, n);
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
}

namespace {

using namespace sph::cuda;

// ------------------------------------------------------------------ launcher
enum class Order { Independent, Sequential };

template <class Kernel, class... Args>
void launch(uint32_t blocks, uint32_t tpb, Order order, Kernel kernel, Args... args) {
    if (order == Order::Sequential) {
        blockDim = {tpb, 1, 1};
        gridDim = {blocks, 1, 1};
        for (uint32_t b = 0; b < blocks; b++)
            for (uint32_t t = 0; t < tpb; t++) {
                blockIdx = {b, 0, 0};
                threadIdx = {t, 0, 0};
                kernel(args...);
            }
        return;
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t b = 0; b < (int64_t)blocks; b++) {
        blockDim = {tpb, 1, 1};
        gridDim = {blocks, 1, 1};
        for (uint32_t t = 0; t < tpb; t++) {
            blockIdx = {(uint32_t)b, 0, 0};
            threadIdx = {t, 0, 0};
            kernel(args...);
        }
    }
}

uint32_t blocks_for(uint32_t n, uint32_t tpb) { return (n + tpb - 1) / tpb; }

// ------------------------------------------------------------------ the simulation state
struct GridArrays {
    std::vector<int32_t> start, end, gidx, aidx;
    NeighborGrid::GridData view(uint32_t count) {
        return NeighborGrid::GridData{std::span<int32_t>(start.data(), start.size()),
                                      std::span<int32_t>(end.data(), end.size()),
                                      std::span<int32_t>(gidx.data(), gidx.size()),
                                      std::span<int32_t>(aidx.data(), aidx.size()), count};
    }
};

struct RefSim {
    Simulation::Parameters P{};
    bool adaptive = false;
    refinement::RefinementParameters R{};
    uint32_t cap = 0, n = 0, nb = 0, frame = 0, next_id = 0;
    std::vector<glm::vec4> pos, vel, acc;
    std::vector<float> rho, rad, h, m;
    std::vector<uint32_t> ids;
    std::vector<glm::vec4> bpos, bcol;
    std::vector<float> bpsi, bvisc, brad;
    NeighborGrid::Grid grid{};
    GridArrays fluid, boundary;
    std::unique_ptr<refinement::RefinementData> rd;
    // checker option (not the reference's behaviour): rebuild the fluid grid after the merge compaction, before the
    // split criterion. The reference evaluates the split criterion on the grid of the step, built before
    // compactParticles moved particles down (AdaptiveSphSimulation.cu:135-160), so a criterion that walks neighbours
    // (vorticity) reads shifted slots; with this option the checker shows what the criterion gives on a valid grid.
    bool fresh_split_grid = false;
    // last refinement pass
    orc_report rep{};
    std::vector<uint32_t> keep_ids, removed_ids, split_ids;

    FluidParticlesData fluid_view() {
        return FluidParticlesData{pos.data(), vel.data(), acc.data(), rho.data(), rad.data(), h.data(), m.data(), n};
    }
    BoundaryParticlesData boundary_view() {
        return BoundaryParticlesData{bpos.data(), bcol.data(), bpsi.data(), bvisc.data(), brad.data(), nb};
    }
    NeighborGrid::Device device() {
        return NeighborGrid::Device{P.domain, grid, fluid.view(n), boundary.view(nb)};
    }
    uint32_t tpb() const { return P.threadsPerBlock; }
};

Simulation::Parameters to_params(const orc_params& p) {
    Simulation::Parameters P{};
    P.domain.min = glm::vec3(p.dmin[0], p.dmin[1], p.dmin[2]);
    P.domain.max = glm::vec3(p.dmax[0], p.dmax[1], p.dmax[2]);
    P.domain.friction = p.friction;
    P.gravity = glm::vec3(p.gravity[0], p.gravity[1], p.gravity[2]);
    P.speedOfSound = p.c0;
    P.restDensity = p.rho0;
    P.restitution = p.restitution;
    P.viscosityConstant = p.alpha;
    P.surfaceTensionConstant = p.sigma;
    P.maxVelocity = p.max_velocity;
    P.baseSmoothingRadius = p.h0;
    P.baseParticleRadius = p.r0;
    P.baseParticleMass = p.m0;
    P.threadsPerBlock = p.threads_per_block ? p.threads_per_block : 256;
    return P;
}

refinement::RefinementParameters to_refine(const orc_refine& r) {
    refinement::RefinementParameters R{};
    R.enabled = r.enabled != 0;
    R.minMassRatio = r.min_mass_ratio;
    R.maxMassRatio = r.max_mass_ratio;
    R.maxParticleCount = r.max_particle_count;
    R.maxBatchRatio = r.max_batch_ratio;
    R.initialCooldown = r.initial_cooldown;
    R.cooldown = r.cooldown;
    R.criterionType = r.criterion == 1u   ? refinement::RefinementParameters::Criterion::Interface
                      : r.criterion == 2u ? refinement::RefinementParameters::Criterion::Vorticity
                                          : refinement::RefinementParameters::Criterion::Velocity;
    R.splitting.epsilon = r.eps;
    R.splitting.alpha = r.alpha;
    R.splitting.centerMassRatio = r.center_ratio;
    R.splitting.vertexMassRatio = r.vertex_ratio;
    R.velocity.split.minimalSpeedThreshold = r.vel_split;
    R.velocity.merge.maximalSpeedThreshold = r.vel_merge;
    R.vorticity.split.minimalVorticityThreshold = r.vort_split;
    R.vorticity.merge.maximalVorticityThreshold = r.vort_merge;
    R.curvature.split.minimalCurvatureThreshold = r.curv_split;
    R.curvature.merge.maximalCurvatureThreshold = r.curv_merge;
    R.interfaceParameters.split.distanceRatioThreshold = r.iface_split;
    R.interfaceParameters.merge.distanceRatioThreshold = r.iface_merge;
    return R;
}

// NeighborGrid::createGrid (NeighborGrid.cu:108-121) with the cell width of SphSimulation.cu:47
void make_grid(RefSim& s) {
    const float cellWidth = 2 * s.P.baseSmoothingRadius * device::constant::wendlandRangeRatio;
    const glm::ivec3 gridSize = glm::ivec3{glm::ceil(s.P.domain.getScale() / cellWidth)};
    s.grid.gridSize = gridSize;
    s.grid.cellSize = s.P.domain.getScale() / glm::vec3{gridSize};
    const size_t cells = (size_t)gridSize.x * gridSize.y * gridSize.z;
    for (GridArrays* g : {&s.fluid, &s.boundary}) {
        g->start.assign(cells, -1);
        g->end.assign(cells, -1);
    }
    s.fluid.gidx.assign(s.cap, 0);
    s.fluid.aidx.assign(s.cap, 0);
}

// NeighborGrid::updateFluid / updateBoundary (NeighborGrid.cu:33-50, 134-150): reset the tables, assign cells, sort
// (key, index) by key (Thrust's radix sort of integer keys is stable), start/end indices.
void update_grid(RefSim& s, bool boundary) {
    GridArrays& g = boundary ? s.boundary : s.fluid;
    const uint32_t count = boundary ? s.nb : s.n;
    std::fill(g.start.begin(), g.start.end(), -1);
    std::fill(g.end.begin(), g.end.end(), -1);
    if (g.gidx.size() < count) {
        g.gidx.resize(count);
        g.aidx.resize(count);
    }
    NeighborGrid::Device dev = s.device();
    NeighborGrid::GridData data = g.view(count);
    glm::vec4* p = boundary ? s.bpos.data() : s.pos.data();
    launch(blocks_for(count, s.tpb()), s.tpb(), Order::Independent, kernel::assignParticlesToCells, p, dev, data);
    std::vector<std::pair<int32_t, int32_t>> kv(count);
    for (uint32_t i = 0; i < count; i++) kv[i] = {g.gidx[i], g.aidx[i]};
    std::stable_sort(kv.begin(), kv.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    for (uint32_t i = 0; i < count; i++) {
        g.gidx[i] = kv[i].first;
        g.aidx[i] = kv[i].second;
    }
    launch(blocks_for(count, s.tpb()), s.tpb(), Order::Independent, kernel::calculateCellStartAndEndIndices, data);
}

// ------------------------------------------------------------------ refinement (AdaptiveSphSimulation.cu)
void reset_refinement(RefSim& s) {
    auto& d = *s.rd;
    thrust::fill(d.split.criterionValues.begin(), d.split.criterionValues.end(), 0.0f);
    thrust::fill(d.split.particlesIdsToSplit.begin(), d.split.particlesIdsToSplit.end(), 0u);
    d.split.particlesSplitCount = 0u;
    thrust::fill(d.merge.criterionValues.begin(), d.merge.criterionValues.end(), 0.0f);
    thrust::fill(d.merge.removalFlags.begin(), d.merge.removalFlags.end(),
                 refinement::RefinementData::RemovalState::Keep);
    thrust::fill(d.merge.prefixSums.begin(), d.merge.prefixSums.end(), 0u);
    thrust::fill(d.merge.eligibleParticles.begin(), d.merge.eligibleParticles.end(), 0u);
    thrust::fill(d.merge.mergeCandidates.begin(), d.merge.mergeCandidates.end(), 0u);
    thrust::fill(d.merge.mergePairs.begin(), d.merge.mergePairs.end(), 0u);
    d.merge.eligibleCount = 0u;
    d.merge.mergeCount = 0u;
    thrust::fill(d.particlesIds.begin(), d.particlesIds.end(), 0u);
}

template <class Gen>
void criterion_values(RefSim& s, float* out, Gen gen) {
    launch(blocks_for(s.n, s.tpb()), s.tpb(), Order::Independent, refinement::getCriterionValues<Gen>, s.fluid_view(),
           out, gen, s.device(), s.P);
}

void merge_pass(RefSim& s) {
    auto& d = *s.rd;
    if (s.n <= 1) return;
    const uint32_t current = s.n;
    const float maxMass = s.R.maxMassRatio * s.P.baseParticleMass;
    float* crit = thrust::raw_pointer_cast(d.merge.criterionValues.data());
    using C = refinement::RefinementParameters::Criterion;
    if (s.R.criterionType == C::Interface)
        criterion_values(s, crit, refinement::interfaceCriterion::MergeCriterionGenerator(maxMass, s.R.interfaceParameters));
    else if (s.R.criterionType == C::Vorticity)
        criterion_values(s, crit, refinement::vorticity::MergeCriterionGenerator(maxMass, s.R.vorticity));
    else
        criterion_values(s, crit, refinement::velocity::MergeCriterionGenerator(maxMass, s.R.velocity.merge));
    refinement::findTopParticlesToMerge(s.fluid_view(), d, s.R, thrust::less<float>{});
    const uint32_t eligible = d.merge.eligibleCount.toHost();
    s.rep.merge_eligible = eligible;
    if (eligible == 0) return;
    launch(blocks_for(eligible, s.tpb()), s.tpb(), Order::Independent, refinement::identifyMergeCandidates,
           s.fluid_view(), refinement::RefinementDataView{d}, s.device(), s.P, s.R);
    launch(blocks_for(current, s.tpb()), s.tpb(), Order::Sequential, refinement::resolveMergePairs,
           refinement::RefinementDataView{d}, current);
    const uint32_t pairs = d.merge.mergeCount.toHost();
    s.rep.merge_pairs = pairs;
    if (pairs == 0) return;
    for (uint32_t k = 0; k < pairs; k++) {
        s.keep_ids.push_back(s.ids[d.merge.mergePairs[2 * k]]);
        s.removed_ids.push_back(s.ids[d.merge.mergePairs[2 * k + 1]]);
    }
    launch(blocks_for(pairs, s.tpb()), s.tpb(), Order::Sequential, refinement::performMerges, s.fluid_view(),
           refinement::RefinementDataView{d}, s.P);
    uint32_t* flags = reinterpret_cast<uint32_t*>(thrust::raw_pointer_cast(d.merge.removalFlags.data()));
    thrust::exclusive_scan(flags, flags + current, d.merge.prefixSums.begin());
    // the ids move with the particles (compactParticles moves kept particles to idx - prefix[idx])
    {
        uint32_t w = 0;
        for (uint32_t i = 0; i < current; i++)
            if (flags[i] == 0) s.ids[w++] = s.ids[i];
    }
    // in order: the in-place moves are then race-free (every destination was already read)
    launch(blocks_for(current, s.tpb()), s.tpb(), Order::Sequential, refinement::compactParticles, s.fluid_view(),
           refinement::RefinementDataView{d}, current);
    s.n = d.particlesCount.toHost();
}

void split_pass(RefSim& s, uint32_t removed) {
    auto& d = *s.rd;
    const float minMass = s.R.minMassRatio * s.P.baseParticleMass;
    if (s.fresh_split_grid) update_grid(s, false);
    float* crit = thrust::raw_pointer_cast(d.split.criterionValues.data());
    using C = refinement::RefinementParameters::Criterion;
    if (s.R.criterionType == C::Interface)
        criterion_values(s, crit,
                         refinement::interfaceCriterion::SplitCriterionGenerator(minMass, s.R.interfaceParameters,
                                                                                 s.R.splitting));
    else if (s.R.criterionType == C::Vorticity)
        criterion_values(s, crit, refinement::vorticity::SplitCriterionGenerator(minMass, s.R.vorticity, s.R.splitting));
    else
        criterion_values(s, crit,
                         refinement::velocity::SplitCriterionGenerator(minMass, s.R.velocity.split, s.R.splitting));
    refinement::findTopParticlesToSplit(s.fluid_view(), d, s.R, thrust::greater<float>{});
    const uint32_t candidates = d.split.particlesSplitCount.toHost();
    s.rep.split_candidates = candidates;
    const uint32_t budget = std::min(candidates, removed / 12);
    s.rep.split_budget = budget;
    if (budget == 0) return;
    const uint32_t before = s.n;
    d.particlesCount = s.n;
    launch(blocks_for(budget, s.tpb()), s.tpb(), Order::Sequential, refinement::splitParticles, s.fluid_view(),
           refinement::RefinementDataView{d}, s.R.splitting, s.R.maxParticleCount);
    s.n = d.particlesCount.toHost();
    const uint32_t done = (s.n - before) / 12;
    for (uint32_t r = 0; r < done; r++) {
        s.split_ids.push_back(s.ids[d.split.particlesIdsToSplit[r]]);
        for (uint32_t k = 0; k < 12; k++) s.ids[before + 12 * r + k] = s.next_id + 12 * r + k;
    }
    s.next_id += 12 * done;
    s.rep.splits = done;
}

void refine(RefSim& s) {
    s.rep = orc_report{};
    s.keep_ids.clear();
    s.removed_ids.clear();
    s.split_ids.clear();
    s.rep.frame = s.frame;
    s.rep.count_before = s.n;
    const uint32_t current = s.n;
    reset_refinement(s);
    merge_pass(s);
    const uint32_t removed = current - s.n;
    s.rep.removed = removed;
    if (removed > 0) split_pass(s, removed);
    s.rep.count_after = s.n;
}

// ------------------------------------------------------------------ one step
void half_kick(RefSim& s, float half_dt) {
    launch(blocks_for(s.n, s.tpb()), s.tpb(), Order::Independent, kernel::halfKickVelocities, s.fluid_view(), s.P,
           half_dt);
}

void densities(RefSim& s) {
    launch(blocks_for(s.n, s.tpb()), s.tpb(), Order::Independent, kernel::computeDensities, s.fluid_view(), s.device());
    launch(blocks_for(s.n, s.tpb()), s.tpb(), Order::Independent, kernel::computeBoundaryDensityContribution,
           s.fluid_view(), s.boundary_view(), s.device());
}

void accelerations(RefSim& s) {
    const uint32_t b = blocks_for(s.n, s.tpb()), t = s.tpb();
    launch(b, t, Order::Independent, kernel::computeExternalAccelerations, s.fluid_view(), s.P);
    launch(b, t, Order::Independent, kernel::computePressureAccelerations, s.fluid_view(), s.device(), s.P);
    if (s.P.viscosityConstant != 0.F)
        launch(b, t, Order::Independent, kernel::computeViscosityAccelerations, s.fluid_view(), s.device(), s.P);
    if (s.P.surfaceTensionConstant != 0.F)
        launch(b, t, Order::Independent, kernel::computeSurfaceTensionAccelerations, s.fluid_view(), s.device(), s.P);
    launch(b, t, Order::Independent, kernel::computeBoundaryPressureAcceleration, s.fluid_view(), s.boundary_view(),
           s.device(), s.P);
    launch(b, t, Order::Independent, kernel::computeBoundaryFrictionAcceleration, s.fluid_view(), s.boundary_view(),
           s.device(), s.P);
}

int step(RefSim& s, float dt) {
    half_kick(s, dt / 2.F);
    launch(blocks_for(s.n, s.tpb()), s.tpb(), Order::Independent, kernel::updatePositions, s.fluid_view(),
           s.P.domain, dt);
    update_grid(s, false);
    densities(s);
    accelerations(s);
    int refined = 0;
    if (s.adaptive && (s.frame == s.R.initialCooldown ||
                       (s.frame > s.R.initialCooldown && s.R.cooldown > 0 && s.frame % s.R.cooldown == 0))) {
        refine(s);
        refined = 1;
    }
    half_kick(s, dt / 2.F);
    s.frame++;
    return refined;
}

}  // namespace

// ------------------------------------------------------------------ C interface for the Python checker
extern "C" {

// StaticBoundaryDomain::generate (StaticBoundaryDomain.cu:76-174); returns the count, writes at most cap particles
uint32_t ref_boundary_generate(const float dmin[3], const float dmax[3], float spacing, float rho0, float h,
                               float* pos4, float* psi, uint32_t cap) {
    Simulation::Parameters::Domain d{};
    d.min = glm::vec3(dmin[0], dmin[1], dmin[2]);
    d.max = glm::vec3(dmax[0], dmax[1], dmax[2]);
    const auto dom = physics::StaticBoundaryDomain::generate(d, spacing, rho0, h);
    const auto& ps = dom.getParticles();
    const uint32_t n = (uint32_t)ps.size();
    for (uint32_t i = 0; i < n && i < cap; i++) {
        std::memcpy(pos4 + 4 * (size_t)i, &ps[i].position, 16);
        psi[i] = ps[i].psi;
    }
    return n;
}

// A simulation in the state the reference's constructor leaves (SphSimulation.cu:28-80): the given positions, zero
// velocities, accelerations = gravity, h0, m0, r0; the boundary particles and their grid. refine may be NULL.
void* ref_sim_create(const orc_params* p, const float* pos4, uint32_t n, const float* bpos4, const float* bpsi,
                     uint32_t nb, const orc_refine* refine_params, uint32_t capacity) {
    auto* s = new RefSim();
    s->P = to_params(*p);
    s->adaptive = refine_params && refine_params->enabled;
    if (s->adaptive) s->R = to_refine(*refine_params);
    s->cap = std::max(s->adaptive ? s->R.maxParticleCount : capacity, std::max(n, 1u));
    s->n = n;
    s->next_id = n;
    const glm::vec4 g(s->P.gravity, 0.F);
    s->pos.assign(s->cap, glm::vec4(0.F));
    s->vel.assign(s->cap, glm::vec4(0.F));
    s->acc.assign(s->cap, g);
    s->rho.assign(s->cap, 0.F);
    s->rad.assign(s->cap, 0.F);
    s->h.assign(s->cap, 0.F);
    s->m.assign(s->cap, 0.F);
    s->ids.assign(s->cap, 0u);
    for (uint32_t i = 0; i < n; i++) {
        s->pos[i] = glm::vec4(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], pos4[4 * i + 3]);
        s->rad[i] = s->P.baseParticleRadius;
        s->h[i] = s->P.baseSmoothingRadius;
        s->m[i] = s->P.baseParticleMass;
        s->ids[i] = i;
    }
    s->nb = nb;
    s->bpos.resize(std::max(nb, 1u));
    s->bpsi.resize(std::max(nb, 1u));
    s->bcol.assign(std::max(nb, 1u), glm::vec4(0.3F, 0.3F, 0.3F, 0.2F));
    s->bvisc.assign(std::max(nb, 1u), s->P.domain.friction);
    s->brad.assign(std::max(nb, 1u), s->P.baseParticleRadius);
    for (uint32_t i = 0; i < nb; i++) {
        s->bpos[i] = glm::vec4(bpos4[4 * i], bpos4[4 * i + 1], bpos4[4 * i + 2], bpos4[4 * i + 3]);
        s->bpsi[i] = bpsi[i];
    }
    s->boundary.gidx.assign(std::max(nb, 1u), 0);
    s->boundary.aidx.assign(std::max(nb, 1u), 0);
    make_grid(*s);
    update_grid(*s, true);
    if (s->adaptive) {
        const uint32_t C = s->R.maxParticleCount;
        s->rd.reset(new refinement::RefinementData{
            .split = {.criterionValues = thrust::device_vector<float>(C),
                      .particlesIdsToSplit = thrust::device_vector<uint32_t>(C),
                      .particlesSplitCount = DeviceValue<uint32_t>::fromHost(0)},
            .merge = {.criterionValues = thrust::device_vector<float>(C),
                      .eligibleParticles = thrust::device_vector<uint32_t>(C),
                      .eligibleCount = DeviceValue<uint32_t>::fromHost(0),
                      .mergeCandidates = thrust::device_vector<uint32_t>(C),
                      .mergePairs = thrust::device_vector<uint32_t>(2 * (size_t)C),
                      .removalFlags = thrust::device_vector<refinement::RefinementData::RemovalState>(C),
                      .prefixSums = thrust::device_vector<uint32_t>(C),
                      .mergeCount = DeviceValue<uint32_t>::fromHost(0)},
            .particlesIds = thrust::device_vector<uint32_t>(C),
            .particlesCount = DeviceValue<uint32_t>::fromHost(n)});
    }
    return s;
}

void ref_sim_destroy(void* h) { delete static_cast<RefSim*>(h); }

int ref_sim_step(void* h, float dt) { return step(*static_cast<RefSim*>(h), dt); }

uint32_t ref_sim_count(void* h) { return static_cast<RefSim*>(h)->n; }
uint32_t ref_sim_frame(void* h) { return static_cast<RefSim*>(h)->frame; }
void ref_set_threads(int n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }
void ref_sim_set_fresh_split_grid(void* h, int on) { static_cast<RefSim*>(h)->fresh_split_grid = on != 0; }

// Any pointer may be NULL. Arrays in the reference's own order (array slots), with the checker's ids.
void ref_sim_read(void* hs, float* pos4, float* vel4, float* acc4, float* rho, float* rad, float* h, float* m,
                  uint32_t* id) {
    RefSim& s = *static_cast<RefSim*>(hs);
    for (uint32_t i = 0; i < s.n; i++) {
        if (pos4) std::memcpy(pos4 + 4 * (size_t)i, &s.pos[i], 16);
        if (vel4) std::memcpy(vel4 + 4 * (size_t)i, &s.vel[i], 16);
        if (acc4) std::memcpy(acc4 + 4 * (size_t)i, &s.acc[i], 16);
        if (rho) rho[i] = s.rho[i];
        if (rad) rad[i] = s.rad[i];
        if (h) h[i] = s.h[i];
        if (m) m[i] = s.m[i];
        if (id) id[i] = s.ids[i];
    }
}

// Replaces the fluid state (all pointers required), with the frame counter and the next id.
void ref_sim_write(void* hs, uint32_t n, const float* pos4, const float* vel4, const float* acc4, const float* rho,
                   const float* rad, const float* h, const float* m, const uint32_t* id, uint32_t frame,
                   uint32_t next_id) {
    RefSim& s = *static_cast<RefSim*>(hs);
    s.n = std::min(n, s.cap);
    for (uint32_t i = 0; i < s.n; i++) {
        std::memcpy(&s.pos[i], pos4 + 4 * (size_t)i, 16);
        std::memcpy(&s.vel[i], vel4 + 4 * (size_t)i, 16);
        std::memcpy(&s.acc[i], acc4 + 4 * (size_t)i, 16);
        s.rho[i] = rho[i];
        s.rad[i] = rad[i];
        s.h[i] = h[i];
        s.m[i] = m[i];
        s.ids[i] = id[i];
    }
    s.frame = frame;
    s.next_id = next_id;
}

// The density and acceleration passes alone, on the current positions (grid, computeDensities + boundary
// contribution, then the acceleration kernels): the kernel-level comparison of one state.
void ref_sim_density_forces(void* hs) {
    RefSim& s = *static_cast<RefSim*>(hs);
    update_grid(s, false);
    densities(s);
    accelerations(s);
}

// Per-particle terms of sumAllNeighbors (Algorithm.cu:234-268), each thread run alone into its own counter, over the
// grid of the last update; returns the total.
uint64_t ref_sim_neighbor_counts(void* hs, uint32_t* counts) {
    RefSim& s = *static_cast<RefSim*>(hs);
    uint64_t total = 0;
    const uint32_t tpb = s.tpb();
#pragma omp parallel for reduction(+ : total) schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)s.n; i++) {
        uint32_t c = 0;
        blockDim = {tpb, 1, 1};
        blockIdx = {(uint32_t)(i / tpb), 0, 0};
        threadIdx = {(uint32_t)(i % tpb), 0, 0};
        kernel::sumAllNeighbors(s.fluid_view(), s.device(), &c);
        if (counts) counts[i] = c;
        total += c;
    }
    return total;
}

// The last refinement pass: counts as in orc_report, and the id lists (keep/removed in pair order, split parents in
// split order). Returns the number of pairs.
uint32_t ref_sim_last_refinement(void* hs, orc_report* rep) {
    RefSim& s = *static_cast<RefSim*>(hs);
    uint32_t *rm = rep->removed_ids, *kp = rep->keep_ids, *sp = rep->split_ids;
    *rep = s.rep;
    rep->removed_ids = rm;
    rep->keep_ids = kp;
    rep->split_ids = sp;
    for (size_t k = 0; k < s.keep_ids.size(); k++) {
        if (kp) kp[k] = s.keep_ids[k];
        if (rm) rm[k] = s.removed_ids[k];
    }
    for (size_t k = 0; k < s.split_ids.size(); k++)
        if (sp) sp[k] = s.split_ids[k];
    return (uint32_t)s.keep_ids.size();
}

}  // extern "C"
