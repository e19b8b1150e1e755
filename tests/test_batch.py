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


@pytest.mark.parametrize("mode", ["auto", "graphs", "segmented"])
def test_batch_matches_alone(mode):
    """Plain frames as per-simulation graphs, as segmented passes, or as the autotuner switches between them while
    it times them: every simulation's state equals its state stepped alone, bit for bit."""
    scenes = _scenes()
    alone = [make_pair(sc)[0] for sc in scenes]
    mixed = [make_pair(sc)[0] for sc in scenes]
    dts = [sc.dt for sc in scenes]
    for _ in range(25):
        for sim, dt in zip(alone, dts):
            sim.update(dt)
    batch = Batch(mixed, mode=mode)
    batch.step(dts, 10)
    batch.step(dts, 15)
    for a, m in zip(alone, mixed):
        assert m.get_fluid_particles_count() == a.get_fluid_particles_count()
        assert_state_bitexact(m.read_state(), a.read_state())
    st = batch.stats()
    assert st["graph_steps"] > 0 and st["eager_steps"] > 0
    assert st["captures"] < st["graph_steps"]
    tn = batch.tuning()
    if mode == "segmented":
        assert tn["segmented_steps"] > 0
    if mode == "graphs":
        assert tn["segmented_steps"] == 0
    if mode == "auto":
        assert len(tn["trials"]) > 0
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


def _sim(sc):
    from adaptivesph_gb300 import create_simulation
    from helpers import boundary_of

    bd = boundary_of(sc)
    cap = sc.refinement.max_particle_count if sc.refinement else sc.positions.shape[0]
    return create_simulation(sc.parameters, sc.positions, None, None, bd, sc.refinement, cap,
                             max(bd.get_particle_count(), 1))


def _oracle(sc):
    import oracle
    from helpers import boundary_of

    bd = boundary_of(sc)
    cap = sc.refinement.max_particle_count if sc.refinement else sc.positions.shape[0]
    return oracle.OracleSim(sc.parameters, sc.positions, bd.positions, bd.psi, sc.refinement, capacity=cap)


def _mix_slice():
    """28 scenes of the 256-scene mix (counts log-uniform in 4k-256k, Morris nu log-uniform in 1e-6..1e-3,
    refinement on the even scenes): the first 28, as generated."""
    from adaptivesph_gb300 import scenes

    return scenes.batched_mix()[:28]


@pytest.mark.parametrize("mode", ["segmented", "auto"])
def test_batched_mix_slice_alone_vs_batch_and_oracle(mode):
    """Each of 28 scenes of the batched mix gives, in one batch with the 27 others, the state it gives alone, bit for
    bit, over 25 frames (refinement frames 10 and 20 included); the 3 smallest (one adaptive) also match the oracle.
    Segmented: every plain frame's density and force passes run as launches shared by the scenes (Morris viscosity,
    one kernel variant); auto: the autotuner's trial configurations during the same frames."""
    mix = _mix_slice()
    counts = [sc.positions.shape[0] for sc in mix]
    assert min(counts) < 16384 and max(counts) > 65536, "uneven counts wanted"
    steps = 25
    alone = [_sim(sc) for sc in mix]
    for sim, sc in zip(alone, mix):
        for _ in range(steps):
            sim.update(sc.dt)
    mixed = [_sim(sc) for sc in mix]
    batch = Batch(mixed, mode=mode)
    batch.step([sc.dt for sc in mix], steps)
    refined = 0
    for a, m, sc in zip(alone, mixed, mix):
        assert m.get_fluid_particles_count() == a.get_fluid_particles_count(), sc.name
        assert_state_bitexact(m.read_state(), a.read_state())
        refined += int(sc.refinement is not None and m.get_fluid_particles_count() != sc.positions.shape[0])
    assert refined > 0, "some adaptive scene must have changed its particle count"
    assert batch.stats()["graph_steps"] > 0
    batch.close()
    order = np.argsort(counts, kind="stable")
    smallest = [int(k) for k in order[:3]]
    if not any(mix[k].refinement is not None for k in smallest):
        smallest[-1] = next(int(k) for k in order if mix[int(k)].refinement is not None)
    for k in smallest:
        sc = mix[k]
        orc = _oracle(sc)
        for _ in range(steps):
            orc.step(sc.dt)
        assert_state_bitexact(mixed[k].read_state(), orc.arrays())
    for s in alone + mixed:
        s.close()


def test_batch_member_update_domain_recaptures():
    """A batch member whose domain shrinks between batch steps (updateDomain, no reallocation of its tables) steps
    on the new grid and walls: the same sequence run alone gives the same state bit for bit."""
    from helpers import boundary_of
    from adaptivesph_gb300.parameters import Domain

    runs = []
    for batched in (False, True):
        scenes_ = _scenes()[:2]  # fresh scenes: update_domain writes the new domain into the scene's parameters
        sims = [make_pair(sc)[0] for sc in scenes_]
        dts = [sc.dt for sc in scenes_]
        batch = Batch(sims) if batched else None

        def advance(k):
            if batch is not None:
                batch.step(dts, k)
            else:
                for sim, dt in zip(sims, dts):
                    for _ in range(k):
                        sim.update(dt)

        advance(12)
        captures0 = batch.stats()["captures"] if batch is not None else 0
        sc = scenes_[0]
        d = sc.parameters.domain
        small = Domain(min=tuple(d.min), max=(d.max[0] * 0.9, d.max[1], d.max[2] * 0.95), friction=d.friction)
        sc_small = small_dam_break()
        sc_small.parameters.domain = small
        sims[0].update_domain(small, boundary_of(sc_small))
        advance(12)
        runs.append([s.read_state() for s in sims])
        if batch is not None:
            assert batch.stats()["captures"] > captures0, "the changed member must be captured again"
            batch.close()
        for s in sims:
            s.close()
    for a, m in zip(runs[0], runs[1]):
        assert_state_bitexact(m, a)
