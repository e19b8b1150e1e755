"""More GPU parity cases through the C ABI: the other refinement criteria, the periodic Taylor-Green box with Morris
viscosity, the CFL step, tiny particle counts (the reference's excluded-cell quirk), an empty boundary and the split
capacity limit. The oracle is the checker; FP32 results are compared bit for bit."""
import dataclasses

import numpy as np
import pytest

from adaptivesph_gb300 import StaticBoundaryDomain, create_simulation, scenes
from adaptivesph_gb300.parameters import Criterion
import oracle
from helpers import (adaptive_refinement, assert_bitexact, assert_state_bitexact, boundary_of, make_pair,
                     small_dam_break)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("criterion", [Criterion.VORTICITY, Criterion.INTERFACE, Criterion.FREE_SURFACE])
def test_criterion_trajectory_bitexact(criterion):
    ref = adaptive_refinement(criterion=criterion, velocity_split_min_speed=2.0, velocity_merge_max_speed=0.1)
    sc = small_dam_break(refinement=ref)
    sim, orc = make_pair(sc)
    sim.record_refinement_ids(True)
    merges = splits = 0
    for k in range(30):
        sim.update(sc.dt)
        if orc.step(sc.dt):
            rep, o = sim.last_refinement(), orc.last_report()
            for key in ("merge_eligible", "merge_pairs", "split_candidates", "split_budget", "splits", "count_after"):
                assert rep[key] == o[key], (k, key, rep[key], o[key])
            assert sim.refinement_ids()["split_ids"].tolist() == o["split_ids"].tolist()
            merges += rep["merge_pairs"]
            splits += rep["splits"]
        assert_state_bitexact(sim.read_state(), orc.arrays())
    assert merges > 0 and splits > 0


def _taylor_green_pair(n=16):
    sc = scenes.taylor_green(n)
    bd = StaticBoundaryDomain.empty(sc.parameters.domain)
    N = sc.positions.shape[0]
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd, None, N, 1)
    orc = oracle.OracleSim(sc.parameters, sc.positions, None, None, None, capacity=N)
    st = sim.read_state()
    st["vel"] = sc.velocities.copy()
    sim.write_state(st, next_id=N)
    a = orc.arrays()
    a["vel"] = sc.velocities.copy()
    orc.load(a, next_id=N)
    return sc, sim, orc


def test_taylor_green_periodic_morris_bitexact():
    sc, sim, orc = _taylor_green_pair()
    ke = []
    for k in range(12):
        sim.update(sc.dt)
        orc.step(sc.dt)
        if k % 4 == 3:
            assert_state_bitexact(sim.read_state(), orc.arrays())
        ke.append(sim.totals()["kinetic_energy"])
    # viscous decay: kinetic energy falls monotonically in a periodic box without forcing
    assert all(b < a for a, b in zip(ke, ke[1:]))
    assert sim.device_errors() == 0


def test_taylor_green_forces_against_fp64():
    sc, sim, orc = _taylor_green_pair()
    for _ in range(3):
        sim.update(sc.dt)
        orc.step(sc.dt)
    from adaptivesph_gb300 import _lib

    sim.run_stages(sc.dt, _lib.STAGE_FORCES)
    orc.integrate(sc.dt)
    orc.grid_build()
    orc.rho[: orc.n] = orc.density32()
    a32 = orc.forces32()
    a64, scale = orc.forces64()
    g = sim.read_state()
    assert_bitexact("acc", g["acc"], a32)
    err = np.abs(g["acc"][:, :3].astype(np.float64) - a64[:, :3]).max(axis=1)
    assert (err / scale).max() <= 1e-5
    rho64 = orc.density64()
    assert (np.abs(g["rho"] - rho64) / rho64).max() <= 1e-5


def test_cfl_step_matches_definition():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    for _ in range(5):
        sim.update(sc.dt)
        orc.step(sc.dt)
    v = orc.export_velocities()[:, :3].astype(np.float64)
    h = orc.arrays()["h"].astype(np.float64)
    want = 0.25 * np.min(h / (sc.parameters.speed_of_sound + np.linalg.norm(v, axis=1)))
    dt = sim.step_cfl(0.25)
    assert dt == pytest.approx(want, rel=1e-6)
    orc.step(dt)
    sim.synchronize()
    assert_state_bitexact(sim.read_state(), orc.arrays())
    # dt_max caps the step
    dt2 = sim.step_cfl(0.25, dt_max=1e-7)
    assert dt2 == np.float32(1e-7)


def _tiny_pair(positions):
    sc = small_dam_break()
    p = dataclasses.replace(sc.parameters)
    pos = np.zeros((len(positions), 4), np.float32)
    pos[:, :3] = np.asarray(positions, np.float32)
    bd = StaticBoundaryDomain.empty(p.domain)
    n = pos.shape[0]
    sim = create_simulation(p, pos, None, None, bd, None, n, 1)
    orc = oracle.OracleSim(p, pos, None, None, None, capacity=n)
    return sc, sim, orc


@pytest.mark.parametrize("positions", [
    [(0.30, 0.30, 0.20)],                            # one particle: its cell is skipped (density 0)
    [(0.30, 0.30, 0.20), (0.31, 0.30, 0.20)],        # two particles in one cell: see each other
    [(0.10, 0.30, 0.20), (0.50, 0.30, 0.20)],        # two cells: both skipped by the reference's quirk
])
def test_tiny_particle_counts_bitexact(positions):
    sc, sim, orc = _tiny_pair(positions)
    for _ in range(4):
        sim.update(sc.dt)
        orc.step(sc.dt)
        assert_state_bitexact(sim.read_state(), orc.arrays())
    info = sim.grid_info()
    assert tuple(info["excluded_cells"]) == orc.excluded()


def test_empty_boundary_bitexact():
    sc = small_dam_break(walls=False)
    sim, orc = make_pair(sc)
    assert sim.get_boundary_particles_count() == 0
    for _ in range(10):
        sim.update(sc.dt)
        orc.step(sc.dt)
    assert_state_bitexact(sim.read_state(), orc.arrays())


def test_split_capacity_limit_bitexact():
    """A fluid capacity only a little above the particle count: splits stop at the capacity, like the oracle."""
    sc0 = small_dam_break()
    n = sc0.positions.shape[0]
    ref = adaptive_refinement(capacity=n + 60)
    sc = small_dam_break(refinement=ref)
    sim, orc = make_pair(sc)
    hit = False
    for k in range(20):
        sim.update(sc.dt)
        if orc.step(sc.dt):
            rep, o = sim.last_refinement(), orc.last_report()
            assert rep["splits"] == o["splits"] and rep["count_after"] == o["count_after"]
            hit |= bool(o["capacity_hit"])
        assert_state_bitexact(sim.read_state(), orc.arrays())
    assert hit, "the scene must reach the capacity"
    assert sim.get_fluid_particles_count() <= n + 60


def test_async_export_overlapping_steps_bitexact():
    """asph_simulation_export_host_async: frame k's copies run while frame k + 1 is enqueued and computed; each
    frame's exported arrays equal the oracle's state of that frame."""
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    n = sc.positions.shape[0]

    def host_set():
        return dict(positions=np.zeros((n, 4), np.float32), velocities=np.zeros((n, 4), np.float32),
                    densities=np.zeros(n, np.float32), radii=np.zeros(n, np.float32), ids=np.zeros(n, np.uint32))

    sets = [host_set(), host_set()]
    want = []

    def check(k):
        got, (pos, vel, rho, rad, ids) = sets[k % 2], want[k]
        assert_bitexact("positions", got["positions"], pos)
        assert_bitexact("velocities", got["velocities"], vel)
        assert_bitexact("densities", got["densities"], rho)
        assert_bitexact("radii", got["radii"], rad)
        assert_bitexact("ids", got["ids"], ids)

    for k in range(8):
        sim.step_async(sc.dt)
        orc.step(sc.dt)
        if k > 0:
            sim.export_wait()
            check(k - 1)
        sim.export_host_async(sets[k % 2])
        o = orc.arrays()
        want.append((o["pos"].copy(), orc.export_velocities().copy(), o["rho"].copy(), o["rad"].copy(),
                     o["id"].copy()))
    sim.export_wait()
    check(7)
    # a synchronous export after asynchronous ones sees the same state
    sync = sim.export_host()
    assert_bitexact("positions", sync["positions"], want[7][0])


def test_dense_walls_bitexact():
    """Walls generated at 1/15 of the fluid spacing, with 2h = 0.104 m reaching past them (they lie 0.05 m outside
    the domain): a particle near a corner of the domain has thousands of wall neighbours in up to ~310 blocks of 32
    members, more than its neighbour row holds after its fluid entries (about a dozen of the 165 particles that see
    walls), so the force pass walks the wall cells for those instead of reading recorded wall entries, while the
    others read theirs. Both must give the oracle's result bit for bit."""
    sc = scenes.dam_break((8, 10, 6), 0.04, seed=13, tank=(0.6, 0.6, 0.4), viscosity=0.01)
    sc = dataclasses.replace(sc, boundary_spacing=0.0027)
    sim, orc = make_pair(sc)
    assert sim.get_boundary_particles_count() > 300_000
    for _ in range(4):
        sim.update(sc.dt)
        orc.step(sc.dt)
    assert_state_bitexact(sim.read_state(), orc.arrays())
    assert sim.device_errors() == 0


@pytest.mark.parametrize("morris", [False, True])
def test_cohesion_bitexact_and_fp64(morris):
    """Surface tension on (computeSurfaceTensionAccelerations, Algorithm.cu:176-221; the reference's configs keep it
    off, and the force kernel is compiled with the term only when it is on): a trajectory bit-exact against the
    oracle, then one force pass against its FP32 and FP64 steps."""
    from adaptivesph_gb300 import _lib
    from adaptivesph_gb300.parameters import ViscosityModel

    sc = small_dam_break()
    p = dataclasses.replace(sc.parameters, surface_tension_constant=2.0)
    if morris:
        p = dataclasses.replace(p, viscosity_model=ViscosityModel.MORRIS, kinematic_viscosity=1e-3)
    sc = dataclasses.replace(sc, parameters=p)
    sim, orc = make_pair(sc)
    for _ in range(6):
        sim.update(sc.dt)
        orc.step(sc.dt)
    assert_state_bitexact(sim.read_state(), orc.arrays())
    sim.run_stages(sc.dt, _lib.STAGE_FORCES)
    orc.integrate(sc.dt)
    orc.grid_build()
    orc.rho[: orc.n] = orc.density32()
    g = sim.read_state()
    assert_bitexact("acc", g["acc"], orc.forces32())
    a64, scale = orc.forces64()
    err = np.abs(g["acc"][:, :3].astype(np.float64) - a64[:, :3]).max(axis=1)
    assert (err / scale).max() <= 1e-5


def test_update_domain_bitexact():
    """Simulation::updateDomain (SphSimulation.cu:122-134; the reference's app calls it when the tank is resized,
    app/App.cpp:369-373): the tank grows in x mid-run, with walls generated for the new tank. The oracle restarts
    from the same state with the new domain and walls; both then run on, bit for bit."""
    from adaptivesph_gb300.parameters import Domain

    sc = small_dam_break()
    _, orc = make_pair(sc)
    bd0 = boundary_of(sc)
    n = sc.positions.shape[0]
    # the boundary capacity leaves room for the larger tank, as the reference's app sizes its buffers up front
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd0, None, n, 2 * bd0.get_particle_count())
    for _ in range(5):
        sim.update(sc.dt)
        orc.step(sc.dt)
    assert_state_bitexact(sim.read_state(), orc.arrays())
    d0 = sc.parameters.domain
    d1 = Domain(min=tuple(d0.min), max=(d0.max[0] + 0.2, d0.max[1], d0.max[2]), friction=d0.friction)
    bd1 = StaticBoundaryDomain.generate(d1, sc.boundary_spacing, sc.parameters.rest_density,
                                       sc.parameters.base_smoothing_radius)
    sim.update_domain(d1, bd1)
    assert sim.get_boundary_particles_count() == bd1.get_particle_count()
    p1 = dataclasses.replace(sc.parameters, domain=d1)
    orc1 = oracle.OracleSim(p1, sc.positions, bd1.positions, bd1.psi, None, capacity=n)
    orc1.load(orc.arrays(), frame=int(orc.state.frame), next_id=int(orc.state.next_id),
              pending_half=float(orc.state.pending_half) if orc.state.has_pending else None)
    for _ in range(8):
        sim.update(sc.dt)
        orc1.step(sc.dt)
    assert_state_bitexact(sim.read_state(), orc1.arrays())
    # the fluid now spreads into the new part of the tank
    assert sim.read_state()["pos"][:, 0].max() <= d1.max[0]


def test_enable_adaptive_refinement_bitexact():
    """Simulation::enableAdaptiveRefinement (AdaptiveSphSimulation.cu:87-90): the frame counter jumps to the initial
    cooldown, so the next step runs a refinement pass; the oracle's counter is set the same way."""
    ref = adaptive_refinement(initial_cooldown=50, cooldown=50)
    sc = small_dam_break(refinement=ref)
    sim, orc = make_pair(sc)
    for _ in range(3):
        sim.update(sc.dt)
        assert not orc.step(sc.dt)
    sim.enable_adaptive_refinement()
    orc.state.frame = ref.initial_cooldown
    sim.update(sc.dt)
    assert orc.step(sc.dt), "the step after enableAdaptiveRefinement must refine"
    rep, o = sim.last_refinement(), orc.last_report()
    for key in ("merge_eligible", "merge_pairs", "split_candidates", "splits", "count_after"):
        assert rep[key] == o[key], (key, rep[key], o[key])
    assert rep["merge_pairs"] + rep["splits"] > 0
    assert_state_bitexact(sim.read_state(), orc.arrays())


@pytest.mark.parametrize("path", ["update", "segmented"])
def test_rows_grow_with_the_particle_count_bitexact(path):
    """The neighbour rows are allocated for the particles present (plus headroom) and grown on demand: a state of
    3.8x the created count written into the simulation is stepped through a captured single-simulation step or a
    segmented batch step; every step equals the oracle's and no particle lies beyond the rows (the kernels flag
    that in the device error word, which update and step check)."""
    from adaptivesph_gb300 import Batch
    sc = small_dam_break()
    sim, orc = make_pair(sc, capacity=12000)
    big = small_dam_break(counts=(20, 24, 16))
    big.parameters = sc.parameters
    bd = boundary_of(big)
    o_big = oracle.OracleSim(sc.parameters, big.positions, bd.positions, bd.psi, None, capacity=12000)
    st = o_big.arrays()
    n = st["pos"].shape[0]
    assert n == 7680 and n > 3 * sc.positions.shape[0]
    sim.write_state(st, frame=3, next_id=n, pending_half=sc.dt / 2)
    orc.load(st, frame=3, next_id=n, pending_half=sc.dt / 2)
    if path == "update":
        for _ in range(6):
            sim.update(sc.dt)
            orc.step(sc.dt)
            assert_state_bitexact(sim.read_state(), orc.arrays())
    else:
        batch = Batch([sim], mode="segmented")
        batch.step([sc.dt], 6)
        for _ in range(6):
            orc.step(sc.dt)
        assert batch.tuning()["segmented_steps"] > 0
        assert_state_bitexact(sim.read_state(), orc.arrays())
        batch.close()
    assert sim.device_errors() == 0


def test_creation_in_place_and_staged_equal():
    """Creation reads the positions and wall records in place where the device reads host memory through the
    host's page tables, and stages them through copies elsewhere (forced here by a test hook) or when the positions
    are not 16-byte aligned: every way gives the same state and the same trajectory, bit for bit."""
    from adaptivesph_gb300 import _lib, create_simulation
    sc = small_dam_break()
    bd = boundary_of(sc)
    L = _lib.load()

    def run(pos):
        sim = create_simulation(sc.parameters, pos, None, None, bd, None, pos.shape[0], bd.get_particle_count())
        first = sim.read_state()
        for _ in range(5):
            sim.update(sc.dt)
        st = sim.read_state()
        sim.close()
        return first, st

    a0, a = run(sc.positions)
    prev = L.asph_debug_host_reads_in_place(0)
    try:
        b0, b = run(sc.positions)
    finally:
        L.asph_debug_host_reads_in_place(prev)
    buf = np.empty(sc.positions.size + 1, np.float32)
    mis = buf[1:].reshape(-1, 4)
    mis[:] = sc.positions
    assert mis.ctypes.data % 16 != 0
    c0, c = run(mis)
    for got in (b0, c0):
        assert_state_bitexact(got, a0)
    for got in (b, c):
        assert_state_bitexact(got, a)
