"""Parity at the benchmark sizes, through the C ABI, bit for bit against the oracle.

* The plain 3D dam break (40x80x40 = 128,000 particles at dx = 0.01 m, walls from StaticBoundaryDomain::generate):
  the whole trajectory of its stated 500 steps from the initial lattice.
* The adaptive dam break of the headline measurement (100x200x50 = 1,000,000 particles at dx = 0.004 m, 503,100
  wall particles, velocity criterion, capacity 4M): the GPU runs it alone to frame 155, where merged particles have
  grown to several h0 and every summation kind occurs (heavy boxes, long rows, ordinary rows); its state then goes
  to the oracle, and both take 6 more frames, one of them a refinement frame. A second simulation built from the
  same input reaches frame 155 with the same state bit for bit (run-to-run determinism at full size).
"""
import numpy as np
import pytest

import oracle
from adaptivesph_gb300 import StaticBoundaryDomain, create_simulation, scenes
from helpers import assert_state_bitexact

pytestmark = pytest.mark.gpu


def _scene_pair(sc, capacity):
    bd = StaticBoundaryDomain.generate(sc.parameters.domain, sc.boundary_spacing, sc.parameters.rest_density,
                                       sc.parameters.base_smoothing_radius)
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd, sc.refinement, capacity,
                            bd.get_particle_count())
    orc = oracle.OracleSim(sc.parameters, sc.positions, bd.positions, bd.psi, sc.refinement, capacity=capacity)
    return sim, orc, bd


def test_plain_dam_break_128k_500_steps_bitexact():
    """The plain dam break at its stated length: 500 fixed-dt steps from the lattice (the app's fixed-dt frame loop,
    app/App.cpp:230), compared bit for bit every 50 steps."""
    sc = scenes.c1_plain()
    sim, orc, _ = _scene_pair(sc, sc.positions.shape[0])
    for k in range(500):
        sim.step_async(sc.dt)
        orc.step(sc.dt)
        if k % 50 == 49:
            sim.synchronize()
            assert_state_bitexact(sim.read_state(), orc.arrays())
    assert sim.device_errors() == 0


def test_totals_run_to_run_bit_identical_128k():
    """FP64 totals come from fixed-order reductions: two simulations from the same input give bit-identical totals
    after 30 steps, and so do repeated reads of one state (many blocks: 128k particles)."""
    sc = scenes.c1_plain()
    totals = []
    for _ in range(2):
        sim, _, _ = _scene_pair(sc, sc.positions.shape[0])
        for _ in range(30):
            sim.step_async(sc.dt)
        sim.synchronize()
        a, b = sim.totals(), sim.totals()
        assert a == b
        totals.append(a)
        sim.close()
    assert totals[0] == totals[1]


def _transfer(sim, orc):
    st = sim.read_state()
    info = sim.state_info()
    orc.load(st, frame=int(info["frame"]), next_id=int(info["next_id"]),
             pending_half=info["pending_half_dt"] if info["has_pending"] else None)
    return st, info


def test_adaptive_dam_break_1m_late_frames_bitexact():
    sc = scenes.c2_adaptive()
    cap = sc.refinement.max_particle_count
    sim, orc, bd = _scene_pair(sc, cap)
    for _ in range(155):
        sim.step_async(sc.dt)
    sim.synchronize()
    st, info = _transfer(sim, orc)
    h0 = np.float32(sc.parameters.base_smoothing_radius)
    assert st["h"].max() > 3 * h0, "merged particles must have grown"

    # every summation kind occurs in the next step (a separate oracle instance: its grid build reorders)
    probe = oracle.OracleSim(sc.parameters, sc.positions, bd.positions, bd.psi, sc.refinement, capacity=cap)
    probe.load(st, frame=int(info["frame"]), next_id=int(info["next_id"]),
               pending_half=info["pending_half_dt"] if info["has_pending"] else None)
    probe.integrate(sc.dt)
    probe.grid_build()
    kinds = np.bincount(probe.sum_kinds(), minlength=3)
    assert kinds.min() > 0, kinds
    del probe

    # run-to-run determinism at full size
    bd2 = StaticBoundaryDomain.generate(sc.parameters.domain, sc.boundary_spacing, sc.parameters.rest_density,
                                        sc.parameters.base_smoothing_radius)
    sim2 = create_simulation(sc.parameters, sc.positions, None, None, bd2, sc.refinement, cap,
                             bd2.get_particle_count())
    for _ in range(155):
        sim2.step_async(sc.dt)
    sim2.synchronize()
    assert_state_bitexact(sim2.read_state(), st)
    sim2.close()

    refined = False
    for _ in range(6):
        sim.step_async(sc.dt)
        sim.synchronize()
        if orc.step(sc.dt):
            refined = True
            rep, o = sim.last_refinement(), orc.last_report()
            for key in ("merge_eligible", "merge_pairs", "split_candidates", "splits", "count_after"):
                assert rep[key] == o[key], (key, rep[key], o[key])
        assert_state_bitexact(sim.read_state(), orc.arrays())
    assert refined, "the frames must include a refinement pass"
    assert sim.device_errors() == 0


def test_adaptive_dam_break_1m_frame_2000_bitexact():
    """The 1M adaptive dam break at the end of its stated 2000 steps: the GPU alone to frame 1996, then the oracle
    takes over the same state and both step to frame 2001 (a refinement frame at 2000 included), bit for bit over all
    particles."""
    sc = scenes.c2_adaptive()
    cap = sc.refinement.max_particle_count
    sim, orc, bd = _scene_pair(sc, cap)
    for _ in range(1996):
        sim.step_async(sc.dt)
    sim.synchronize()
    _transfer(sim, orc)
    refined = False
    for _ in range(5):
        sim.step_async(sc.dt)
        sim.synchronize()
        if orc.step(sc.dt):
            refined = True
            rep, o = sim.last_refinement(), orc.last_report()
            for key in ("merge_eligible", "merge_pairs", "split_candidates", "splits", "count_after"):
                assert rep[key] == o[key], (key, rep[key], o[key])
        assert_state_bitexact(sim.read_state(), orc.arrays())
    assert refined, "the frames must include a refinement pass"
    assert sim.device_errors() == 0
    sim.close()


def test_taylor_green_128_cubed_bitexact_and_fp64():
    """The periodic Taylor-Green vortex at 128^3 = 2,097,152 particles (Morris viscosity, Re = 100): two frames
    bit-exact against the oracle over the whole state, then the third frame's densities and accelerations bit-exact
    against the oracle's FP32 step and within 1e-5 of its FP64 step (density relative; force relative to the
    magnitude the FP32 sum carries)."""
    from adaptivesph_gb300 import _lib

    sc = scenes.taylor_green(128)
    n = sc.positions.shape[0]
    bd = StaticBoundaryDomain.empty(sc.parameters.domain)
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd, None, n, 1)
    orc = oracle.OracleSim(sc.parameters, sc.positions, None, None, None, capacity=n)
    st = sim.read_state()
    st["vel"] = sc.velocities.copy()
    sim.write_state(st, next_id=n)
    a = orc.arrays()
    a["vel"] = sc.velocities.copy()
    orc.load(a, next_id=n)
    for _ in range(2):
        sim.update(sc.dt)
        orc.step(sc.dt)
    assert_state_bitexact(sim.read_state(), orc.arrays())
    sim.run_stages(sc.dt, _lib.STAGE_FORCES)
    orc.integrate(sc.dt)
    orc.grid_build()
    orc.rho[: orc.n] = orc.density32()
    g = sim.read_state()
    np.testing.assert_array_equal(g["rho"].view(np.uint32), orc.rho[: orc.n].view(np.uint32))
    np.testing.assert_array_equal(g["acc"].view(np.uint32), orc.forces32().view(np.uint32))
    rho64 = orc.density64()
    assert (np.abs(g["rho"] - rho64) / rho64).max() <= 1e-5
    a64, scale = orc.forces64()
    err = np.abs(g["acc"][:, :3].astype(np.float64) - a64[:, :3]).max(axis=1)
    assert (err / scale).max() <= 1e-5
    assert sim.device_errors() == 0
