// server.cpp — serving loop over the C ABI: scene requests arrive at any time, are admitted first come first served
// while their device memory fits a budget (capacity included, so split headroom is reserved up front), run
// together with every other admitted request (their steps overlap on the device through the batch machinery of
// simulation.cu), and retire when their step count is reached: the particles are copied to host memory, the
// simulation is destroyed and its memory returns to the budget. No reference counterpart; the reference's app runs
// one scene at a time (app/App.cpp:191-251).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/asph.h"
#include "batch_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    asph_parameters params{};
    bool adaptive = false;
    asph_refinement_parameters refine{};
    std::vector<float> positions;
    std::vector<asph_boundary_particle> boundary;
    uint32_t capacity = 0;
    float dt = 0.0f;
    uint32_t steps = 0;
    float wall_spacing = 0.0f;   // > 0: walls generated on the GPU at admission
    uint32_t wall_count = 0;     // their count (known at submission from the lattice loops)
    uint64_t bytes = 0;  // estimated device memory

    uint32_t state = ASPH_REQUEST_QUEUED;
    asph_simulation* sim = nullptr;
    asph::SceneGraph* graph = nullptr;
    uint32_t done = 0;
    double t_submit = 0.0, t_admit = 0.0, t_finish = 0.0;
    asph_status error = ASPH_OK;
    std::string message;
    // results, after retirement
    uint32_t count = 0;
    std::vector<float> pos, vel, rho, rad;
    std::vector<uint32_t> ids;
};

void release(Request& r) {
    if (r.graph) asph::scene_graph_free(r.graph);
    r.graph = nullptr;
    if (r.sim) asph_simulation_destroy(r.sim);
    r.sim = nullptr;
}

}  // namespace

struct asph_server {
    uint64_t budget = 0, used = 0;
    uint32_t max_active = 0;
    uint64_t next_ticket = 1;
    Clock::time_point t0 = Clock::now();
    std::deque<Request*> queue;                          // waiting, in arrival order
    std::vector<Request*> active;                        // admitted and running
    std::map<uint64_t, std::unique_ptr<Request>> all;    // every request not yet taken
    asph::AdvanceStats stats;
    // Submissions, status and stats may come from other threads than the one polling: every change of the queue,
    // the active list, a request's state and the budget is made under this lock (the polling thread alone changes
    // the active list, so it reads it without the lock).
    mutable std::mutex lock;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Starts the request's simulation. On failure the request is marked failed and holds no device memory.
void admit(asph_server* sv, Request* r) {
    r->t_admit = sv->now();
    asph_simulation* sim = nullptr;
    const uint32_t n = (uint32_t)(r->positions.size() / 4);
    asph_status st =
        r->wall_spacing > 0.0f
            ? asph_simulation_create_with_walls(&r->params, r->positions.data(), n, nullptr, nullptr, r->wall_spacing,
                                                r->adaptive ? &r->refine : nullptr, r->capacity, r->wall_count, &sim)
            : asph_simulation_create(&r->params, r->positions.data(), n, nullptr, nullptr,
                                     r->boundary.empty() ? nullptr : r->boundary.data(), (uint32_t)r->boundary.size(),
                                     r->adaptive ? &r->refine : nullptr, r->capacity, (uint32_t)r->boundary.size(),
                                     &sim);
    if (st == ASPH_OK) {
        r->graph = asph::scene_graph_new();
        if (!r->graph) st = ASPH_ERR_OUT_OF_MEMORY;
    }
    if (st != ASPH_OK) {
        if (sim) asph_simulation_destroy(sim);
        std::lock_guard<std::mutex> g(sv->lock);
        r->state = ASPH_REQUEST_FAILED;
        r->error = st;
        r->message = asph_last_error();
        r->t_finish = sv->now();
        return;
    }
    std::lock_guard<std::mutex> g(sv->lock);
    r->sim = sim;
    r->state = ASPH_REQUEST_ACTIVE;
    sv->used += r->bytes;
    sv->active.push_back(r);
    // the positions are on the device now
    std::vector<float>().swap(r->positions);
}

// Copies a finished request's particles to host memory and returns its device memory to the budget. Called with
// the server's lock held.
void retire(asph_server* sv, Request* r) {
    uint32_t n = 0;
    asph_status st = asph_simulation_fluid_count(r->sim, &n);
    if (st == ASPH_OK) {
        r->count = n;
        r->pos.resize(4 * (size_t)n);
        r->vel.resize(4 * (size_t)n);
        r->rho.resize(n);
        r->rad.resize(n);
        r->ids.resize(n);
        st = asph_simulation_export_host(r->sim, r->pos.data(), r->vel.data(), r->rho.data(), r->rad.data(),
                                         r->ids.data(), n);
    }
    r->state = st == ASPH_OK ? ASPH_REQUEST_DONE : ASPH_REQUEST_FAILED;
    if (st != ASPH_OK) {
        r->error = st;
        r->message = asph_last_error();
    }
    r->t_finish = sv->now();
    release(*r);
    sv->used -= r->bytes;
}

}  // namespace

extern "C" {

asph_status asph_server_create(uint64_t memory_budget_bytes, uint32_t max_active, asph_server** out) {
    if (!out) return ASPH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (memory_budget_bytes == 0) return ASPH_ERR_INVALID_ARGUMENT;
    asph_server* sv = new (std::nothrow) asph_server();
    if (!sv) return ASPH_ERR_OUT_OF_MEMORY;
    sv->budget = memory_budget_bytes;
    sv->max_active = max_active ? max_active : 1024u;
    *out = sv;
    return ASPH_OK;
}

void asph_server_destroy(asph_server* sv) {
    if (!sv) return;
    for (auto& kv : sv->all) release(*kv.second);
    delete sv;
}

asph_status asph_server_submit(asph_server* sv, const asph_request* rq, uint64_t* ticket) {
    if (!sv || !rq || !ticket) return ASPH_ERR_INVALID_ARGUMENT;
    if (rq->count > 0 && !rq->positions) return ASPH_ERR_INVALID_ARGUMENT;
    if (rq->boundary_count > 0 && !rq->boundary) return ASPH_ERR_INVALID_ARGUMENT;
    if (!(rq->delta_time == rq->delta_time)) return ASPH_ERR_INVALID_ARGUMENT;
    std::unique_ptr<Request> r(new (std::nothrow) Request());
    if (!r) return ASPH_ERR_OUT_OF_MEMORY;
    r->params = rq->parameters;
    r->adaptive = rq->refinement && rq->refinement->enabled;
    if (r->adaptive) r->refine = *rq->refinement;
    r->positions.assign(rq->positions, rq->positions + 4 * (size_t)rq->count);
    if (rq->boundary_count) r->boundary.assign(rq->boundary, rq->boundary + rq->boundary_count);
    r->capacity = rq->max_fluid_capacity;
    r->dt = rq->delta_time;
    r->steps = rq->steps;
    uint32_t nb = rq->boundary_count;
    if (rq->boundary_count == 0 && rq->wall_spacing > 0.0f) {
        r->wall_spacing = rq->wall_spacing;
        asph_status sw = asph_boundary_generate_gpu(&rq->parameters.domain, rq->wall_spacing,
                                                    rq->parameters.rest_density,
                                                    rq->parameters.base_smoothing_radius, nullptr, 0, &r->wall_count);
        if (sw != ASPH_OK) return sw;
        nb = r->wall_count;
    }
    asph_status st = asph_estimate_device_bytes(&r->params, rq->count, nb, r->adaptive ? &r->refine : nullptr,
                                                r->capacity, nb, &r->bytes);
    if (st != ASPH_OK) return st;
    std::lock_guard<std::mutex> g(sv->lock);
    if (r->bytes > sv->budget) return ASPH_ERR_CAPACITY;  // could never be admitted
    r->ticket = sv->next_ticket++;
    r->t_submit = sv->now();
    *ticket = r->ticket;
    sv->queue.push_back(r.get());
    sv->all[r->ticket] = std::move(r);
    return ASPH_OK;
}

asph_status asph_server_poll(asph_server* sv, uint32_t max_steps, uint32_t* outstanding) {
    if (!sv) return ASPH_ERR_INVALID_ARGUMENT;
    std::vector<Request*> admitted;
    {
        std::lock_guard<std::mutex> g(sv->lock);
        // first come, first served: admission stops at the first request that does not fit
        uint64_t reserve = sv->used;
        while (!sv->queue.empty() && sv->active.size() + admitted.size() < sv->max_active &&
               reserve + sv->queue.front()->bytes <= sv->budget) {
            reserve += sv->queue.front()->bytes;
            admitted.push_back(sv->queue.front());
            sv->queue.pop_front();
        }
    }
    for (Request* r : admitted) admit(sv, r);
    // advance every active request by up to max_steps
    const size_t S = sv->active.size();
    if (S > 0) {
        std::vector<asph_simulation*> sims(S);
        std::vector<asph::SceneGraph*> graphs(S);
        std::vector<float> dts(S);
        std::vector<uint32_t> left(S), before(S);
        for (size_t k = 0; k < S; k++) {
            Request* r = sv->active[k];
            sims[k] = r->sim;
            graphs[k] = r->graph;
            dts[k] = r->dt;
            left[k] = std::min(max_steps ? max_steps : r->steps, r->steps - r->done);
            before[k] = left[k];
        }
        asph::AdvanceStats adv{};
        const asph_status st = asph::advance_scenes(sims.data(), graphs.data(), dts.data(), left.data(), S, adv);
        std::vector<Request*> still;
        std::lock_guard<std::mutex> g(sv->lock);
        sv->stats.graph_steps += adv.graph_steps;
        sv->stats.eager_steps += adv.eager_steps;
        sv->stats.captures += adv.captures;
        for (size_t k = 0; k < S; k++) {
            Request* r = sv->active[k];
            r->done += before[k] - left[k];
            if (st != ASPH_OK && left[k] > 0) {
                // the advance stopped: fail what did not finish, keep the device consistent for the others
                r->state = ASPH_REQUEST_FAILED;
                r->error = st;
                r->message = asph_last_error();
                r->t_finish = sv->now();
                release(*r);
                sv->used -= r->bytes;
            } else if (r->done >= r->steps) {
                retire(sv, r);
            } else {
                still.push_back(r);
            }
        }
        sv->active.swap(still);
    }
    if (outstanding) {
        std::lock_guard<std::mutex> g(sv->lock);
        *outstanding = (uint32_t)(sv->queue.size() + sv->active.size());
    }
    return ASPH_OK;
}

asph_status asph_server_status(asph_server* sv, uint64_t ticket, asph_request_status* out) {
    if (!sv || !out) return ASPH_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->lock);
    auto it = sv->all.find(ticket);
    if (it == sv->all.end()) return ASPH_ERR_INVALID_ARGUMENT;
    const Request& r = *it->second;
    std::memset(out, 0, sizeof(*out));
    out->state = r.state;
    out->steps_done = r.done;
    out->steps = r.steps;
    out->count = r.count;
    out->error = r.error;
    out->device_bytes = r.bytes;
    out->submit_s = r.t_submit;
    out->admit_s = r.t_admit;
    out->finish_s = r.t_finish;
    return ASPH_OK;
}

asph_status asph_server_take(asph_server* sv, uint64_t ticket, float* positions, float* velocities, float* densities,
                             float* radii, uint32_t* ids, uint32_t capacity) {
    if (!sv) return ASPH_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->lock);
    auto it = sv->all.find(ticket);
    if (it == sv->all.end()) return ASPH_ERR_INVALID_ARGUMENT;
    Request& r = *it->second;
    if (r.state == ASPH_REQUEST_FAILED) {
        const asph_status e = r.error;
        sv->all.erase(it);
        return e != ASPH_OK ? e : ASPH_ERR_CUDA;
    }
    if (r.state != ASPH_REQUEST_DONE) return ASPH_ERR_INVALID_ARGUMENT;
    if (capacity < r.count) return ASPH_ERR_CAPACITY;
    const size_t n = r.count;
    if (positions) std::memcpy(positions, r.pos.data(), sizeof(float) * 4 * n);
    if (velocities) std::memcpy(velocities, r.vel.data(), sizeof(float) * 4 * n);
    if (densities) std::memcpy(densities, r.rho.data(), sizeof(float) * n);
    if (radii) std::memcpy(radii, r.rad.data(), sizeof(float) * n);
    if (ids) std::memcpy(ids, r.ids.data(), sizeof(uint32_t) * n);
    sv->all.erase(it);
    return ASPH_OK;
}

asph_status asph_server_stats(const asph_server* sv, uint64_t* used_bytes, uint32_t* queued, uint32_t* active,
                              uint64_t* graph_steps, uint64_t* eager_steps) {
    if (!sv) return ASPH_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->lock);
    if (used_bytes) *used_bytes = sv->used;
    if (queued) *queued = (uint32_t)sv->queue.size();
    if (active) *active = (uint32_t)sv->active.size();
    if (graph_steps) *graph_steps = sv->stats.graph_steps;
    if (eager_steps) *eager_steps = sv->stats.eager_steps;
    return ASPH_OK;
}

}  // extern "C"
