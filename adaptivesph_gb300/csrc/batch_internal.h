// batch_internal.h — the batch machinery of simulation.cu shared with the serving loop (server.cpp); not part of
// the C ABI.
#pragma once

#include <cstddef>
#include <cstdint>

#include "../../include/asph.h"

namespace asph {

// Per-simulation cache of captured steps.
struct SceneGraph;
SceneGraph* scene_graph_new();
void scene_graph_free(SceneGraph* g);

struct AdvanceStats {
    uint64_t graph_steps = 0, eager_steps = 0, captures = 0;
};

// Advances sims[k] by left[k] steps of dts[k] (left[k] is counted down to 0), the simulations' steps overlapping on
// the device; returns after all of them finished and their device error words were checked.
asph_status advance_scenes(asph_simulation* const* sims, SceneGraph* const* graphs, const float* dts, uint32_t* left,
                           size_t count, AdvanceStats& stats);

}  // namespace asph
