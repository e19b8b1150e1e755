"""Batches: simulations stepped together give exactly the results they give alone (plain and adaptive, graphs
replayed across refinement frames and particle-count changes)."""
import numpy as np
import pytest

from adaptivesph_gb300 import Batch
from helpers import adaptive_refinement, assert_state_bitexact, make_pair, small_dam_break

pytestmark = pytest.mark.gpu


def _scenes():
    return [
        small_dam_break(),                                                    # plain
        small_dam_break(counts=(8, 12, 8), seed=3),                           # plain, smaller
        small_dam_break(refinement=adaptive_refinement()),                    # adaptive
        small_dam_break(counts=(12, 16, 8), seed=5, refinement=adaptive_refinement(cooldown=4)),
    ]


def test_batch_matches_alone():
    scenes = _scenes()
    alone = [make_pair(sc)[0] for sc in scenes]
    mixed = [make_pair(sc)[0] for sc in scenes]
    dts = [sc.dt for sc in scenes]
    for _ in range(25):
        for sim, dt in zip(alone, dts):
            sim.update(dt)
    batch = Batch(mixed)
    batch.step(dts, 10)
    batch.step(dts, 15)
    for a, m in zip(alone, mixed):
        assert m.get_fluid_particles_count() == a.get_fluid_particles_count()
        assert_state_bitexact(m.read_state(), a.read_state())
    st = batch.stats()
    assert st["graph_steps"] > 0 and st["eager_steps"] > 0
    assert st["captures"] < st["graph_steps"]
    batch.close()


def test_batch_matches_oracle():
    scenes = _scenes()[2:]
    pairs = [make_pair(sc) for sc in scenes]
    batch = Batch([p[0] for p in pairs])
    batch.step([sc.dt for sc in scenes], 20)
    for (sim, orc), sc in zip(pairs, scenes):
        for _ in range(20):
            orc.step(sc.dt)
        assert_state_bitexact(sim.read_state(), orc.arrays())
