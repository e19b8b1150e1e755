"""GPU parity: the CUDA pipeline against the oracle on identical state, through the C ABI.

Integer outputs (cell keys, sorted order, cell tables, excluded cells, neighbour counts) must be bit-exact. The
CUDA kernels perform the oracle's FP32 operations in the same order, so FP32 outputs are compared bit for bit
as well; in addition FP32 results are checked against the FP64 restatement:
  density: |rho32 - rho64| <= 1e-5 * rho64;
  forces:  |a32 - a64| <= 1e-5 * S, S = |g| + sum_j |pair terms| (FP64), the magnitude the FP32 sum carries
           (pressure terms nearly cancel in the bulk, so |a| itself is not a meaningful scale).
"""
import numpy as np
import pytest

from adaptivesph_gb300 import _lib, scenes
from helpers import (adaptive_refinement, assert_bitexact, assert_state_bitexact, make_pair, small_dam_break)

pytestmark = pytest.mark.gpu

DENSITY_RTOL = 1e-5
FORCE_RTOL = 1e-5


def _advance(sim, orc, dt, steps):
    for _ in range(steps):
        sim.update(dt)
        orc.step(dt)


def test_initial_state_matches():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    assert_state_bitexact(sim.read_state(), orc.arrays())


def test_integrate_bitexact():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 3)
    sim.run_stages(sc.dt, _lib.STAGE_INTEGRATE)
    orc.integrate(sc.dt)
    assert_state_bitexact(sim.read_state(), orc.arrays(), keys=("pos", "vel", "id"))


def test_grid_keys_order_and_tables_bitexact():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 3)
    sim.run_stages(sc.dt, _lib.STAGE_GRID)
    orc.integrate(sc.dt)
    orc.grid_build()
    g = sim.read_state()
    o = orc.arrays()
    assert_state_bitexact(g, o, keys=("pos", "vel", "acc", "rad", "h", "m", "id"))
    keys, start, end = sim.read_grid()
    assert_bitexact("keys", keys, orc.sorted_keys())
    assert_bitexact("cell_start", start, orc.cstart)
    assert_bitexact("cell_end", end, orc.cend)
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    info = sim.grid_info()
    assert tuple(info["excluded_cells"]) == orc.excluded()
    assert tuple(info["boundary_excluded_cells"]) == (int(orc.boundary.ex[0]), int(orc.boundary.ex[1]))


def test_density_bitexact_and_fp64():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 5)
    sim.run_stages(sc.dt, _lib.STAGE_DENSITY)
    orc.integrate(sc.dt)
    orc.grid_build()
    r32 = orc.density32()
    r64 = orc.density64()
    g = sim.read_state()
    assert_bitexact("rho", g["rho"], r32)
    rel = np.abs(g["rho"].astype(np.float64) - r64) / r64
    assert rel.max() <= DENSITY_RTOL, rel.max()


def test_forces_bitexact_and_fp64():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 5)
    sim.run_stages(sc.dt, _lib.STAGE_FORCES)
    orc.integrate(sc.dt)
    orc.grid_build()
    orc.rho[: orc.n] = orc.density32()
    a32 = orc.forces32()
    a64, scale = orc.forces64()
    g = sim.read_state()
    assert_bitexact("acc", g["acc"], a32)
    err = np.abs(g["acc"][:, :3].astype(np.float64) - a64[:, :3]).max(axis=1)
    assert (err / scale).max() <= FORCE_RTOL, (err / scale).max()


def _mixed_h_state(sim, orc, sc, seed=7):
    """State with smoothing lengths h0, 1.5 h0, 3 h0 and 6 h0 mixed at random: large boxes (heavy particles, one
    warp each walking the cells) and long neighbour rows (one warp each over the row) both occur."""
    st = sim.read_state()
    rng = np.random.default_rng(seed)
    h0 = np.float32(sc.parameters.base_smoothing_radius)
    choice = rng.choice(4, size=st["h"].shape[0], p=[0.85, 0.08, 0.05, 0.02])
    st["h"] = (h0 * np.array([1.0, 1.5, 3.0, 6.0], np.float32)[choice]).astype(np.float32)
    sim.write_state(st, frame=5, next_id=int(st["id"].max()) + 1, pending_half=sc.dt / 2)
    orc.load(st, frame=5, next_id=int(st["id"].max()) + 1, pending_half=sc.dt / 2)
    return st


def test_mixed_smoothing_lengths_bitexact():
    sc = small_dam_break(counts=(16, 24, 16), dx=0.02, tank=(0.7, 0.7, 0.5))
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 2)
    _mixed_h_state(sim, orc, sc)
    sim.run_stages(sc.dt, _lib.STAGE_FORCES)
    orc.integrate(sc.dt)
    orc.grid_build()
    kinds = np.bincount(orc.sum_kinds(), minlength=3)
    orc.rho[: orc.n] = orc.density32()
    g = sim.read_state()
    assert_bitexact("rho", g["rho"], orc.rho[: orc.n])
    assert_bitexact("acc", g["acc"], orc.forces32())
    assert kinds[1] > 0 and kinds[2] > 0, ("heavy boxes and long rows must both occur", kinds)
    a64, scale = orc.forces64()
    err = np.abs(g["acc"][:, :3].astype(np.float64) - a64[:, :3]).max(axis=1)
    assert (err / scale).max() <= FORCE_RTOL, (err / scale).max()


def test_neighbor_counts_exact():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 4)
    got = sim.neighbor_counts()
    want = orc.neighbor_counts()
    assert_bitexact("neighbour counts", got, want)
    avg = sim.calculate_average_neighbor_count()
    assert avg == pytest.approx(np.float32(want.sum(dtype=np.uint64)) / np.float32(len(want)), rel=0, abs=0)


@pytest.mark.parametrize("steps", [40])
def test_plain_trajectory_bitexact(steps):
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    for k in range(steps):
        sim.update(sc.dt)
        orc.step(sc.dt)
        if k % 10 == 9 or k == steps - 1:
            assert_state_bitexact(sim.read_state(), orc.arrays())
    assert sim.device_errors() == 0


def test_export_velocities_include_pending_kick():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 6)
    out = sim.export_host()
    o = orc.arrays()
    assert_bitexact("ids", out["ids"], o["id"])
    assert_bitexact("positions", out["positions"], o["pos"])
    assert_bitexact("velocities", out["velocities"], orc.export_velocities())
    assert_bitexact("densities", out["densities"], o["rho"])
    assert_bitexact("radii", out["radii"], o["rad"])


def test_totals_fp64():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 6)
    t = sim.totals()
    want = orc.totals()
    assert t["count"] == orc.n
    assert t["mass"] == pytest.approx(want[0], rel=1e-12)
    # a momentum component can be a near-cancellation: its error scales with sum m|v|, not with the net value
    v = orc.export_velocities()[:, :3].astype(np.float64)
    scale = (orc.arrays()["m"].astype(np.float64)[:, None] * np.abs(v)).sum(axis=0)
    np.testing.assert_array_less(np.abs(np.asarray(t["momentum"]) - want[1:4]), 1e-12 * scale + 1e-300)
    assert t["kinetic_energy"] == pytest.approx(want[4], rel=1e-9)


def test_density_info_matches_definition():
    sc = small_dam_break()
    sim, orc = make_pair(sc)
    _advance(sim, orc, sc.dt, 6)
    info = sim.get_density_info(0.01)
    rho = orc.arrays()["rho"]
    ratio = rho / np.float32(1000.0) - np.float32(1.0)
    assert info.min_density == rho.min() and info.max_density == rho.max()
    assert info.under_density_count == int((ratio < -0.01).sum())
    assert info.normal_density_count == int(((ratio >= -0.01) & (ratio <= 0.01)).sum())
    assert info.over_density_count == int((ratio > 0.01).sum())
    assert info.average_density == pytest.approx(rho.astype(np.float64).mean(), rel=1e-6)


def test_adaptive_velocity_trajectory_bitexact():
    ref = adaptive_refinement()
    sc = small_dam_break(refinement=ref)
    sim, orc = make_pair(sc)
    sim.record_refinement_ids(True)
    saw_merge = saw_split = False
    for k in range(30):
        sim.update(sc.dt)
        refined = orc.step(sc.dt)
        if refined:
            rep = sim.last_refinement()
            o = orc.last_report()
            for key in ("merge_eligible", "merge_pairs", "removed", "split_candidates", "split_budget", "splits",
                        "count_after"):
                assert rep[key] == o[key], (k, key, rep[key], o[key])
            ids = sim.refinement_ids()
            assert sorted(ids["keep_ids"].tolist()) == sorted(o["keep_ids"].tolist())
            assert sorted(ids["removed_ids"].tolist()) == sorted(o["removed_ids"].tolist())
            assert ids["split_ids"].tolist() == o["split_ids"].tolist()
            saw_merge |= rep["merge_pairs"] > 0
            saw_split |= rep["splits"] > 0
        assert_state_bitexact(sim.read_state(), orc.arrays())
    assert saw_merge and saw_split, "the scene must exercise both merging and splitting"


def test_refinement_with_large_smoothing_lengths_bitexact():
    """A refinement frame on a state with h up to 6 h0: large merge-candidate boxes go to the warp kernel, whose
    nearest-candidate choice must equal the oracle's sequential scan."""
    ref = adaptive_refinement(max_mass_ratio=64.0)
    sc = small_dam_break(counts=(16, 24, 16), dx=0.02, tank=(0.7, 0.7, 0.5), refinement=ref)
    sim, orc = make_pair(sc)
    sim.record_refinement_ids(True)
    _advance(sim, orc, sc.dt, 2)
    st = sim.read_state()
    rng = np.random.default_rng(3)
    h0 = np.float32(sc.parameters.base_smoothing_radius)
    choice = rng.choice(4, size=st["h"].shape[0], p=[0.7, 0.1, 0.1, 0.1])
    st["h"] = (h0 * np.array([1.0, 2.0, 4.5, 6.0], np.float32)[choice]).astype(np.float32)
    st["m"] = (st["m"] * np.array([1.0, 8.0, 24.0, 40.0], np.float32)[choice]).astype(np.float32)
    nid = int(st["id"].max()) + 1
    sim.write_state(st, frame=6, next_id=nid, pending_half=sc.dt / 2)
    orc.load(st, frame=6, next_id=nid, pending_half=sc.dt / 2)
    sim.update(sc.dt)
    assert orc.step(sc.dt), "the frame must run the refinement pass"
    rep = sim.last_refinement()
    o = orc.last_report()
    for key in ("merge_eligible", "merge_pairs", "removed", "split_candidates", "split_budget", "splits",
                "count_after"):
        assert rep[key] == o[key], (key, rep[key], o[key])
    assert rep["merge_pairs"] > 0
    ids = sim.refinement_ids()
    assert sorted(ids["keep_ids"].tolist()) == sorted(o["keep_ids"].tolist())
    assert sorted(ids["removed_ids"].tolist()) == sorted(o["removed_ids"].tolist())
    assert_state_bitexact(sim.read_state(), orc.arrays())


def test_every_summation_kind_bitexact():
    """A dense lattice (h = 2.6 dx, so sub-cells hold over 100 members) with mostly 3 h0 particles: heavy boxes,
    overflowed rows (more than 128 entries), long rows and ordinary particles all occur in one pass."""
    sc = scenes.dam_break((24, 24, 24), 0.02, seed=11, tank=(0.7, 0.7, 0.7), h_ratio=2.6)
    sim, orc = make_pair(sc)
    st = sim.read_state()
    rng = np.random.default_rng(7)
    h0 = np.float32(sc.parameters.base_smoothing_radius)
    choice = rng.choice(4, size=st["h"].shape[0], p=[0.3, 0.1, 0.5, 0.1])
    st["h"] = (h0 * np.array([1.0, 2.0, 3.0, 1.5], np.float32)[choice]).astype(np.float32)
    sim.write_state(st, frame=5, next_id=int(st["id"].max()) + 1, pending_half=sc.dt / 2)
    orc.load(st, frame=5, next_id=int(st["id"].max()) + 1, pending_half=sc.dt / 2)
    sim.run_stages(sc.dt, _lib.STAGE_FORCES)
    orc.integrate(sc.dt)
    orc.grid_build()
    kinds = np.bincount(orc.sum_kinds(), minlength=3)
    entries = orc.list_entries()
    assert kinds.min() > 10 and (entries > 256).sum() > 10, (kinds, int((entries > 256).sum()))
    orc.rho[: orc.n] = orc.density32()
    g = sim.read_state()
    assert_bitexact("rho", g["rho"], orc.rho[: orc.n])
    assert_bitexact("acc", g["acc"], orc.forces32())
    a64, scale = orc.forces64()
    err = np.abs(g["acc"][:, :3].astype(np.float64) - a64[:, :3]).max(axis=1)
    assert (err / scale).max() <= FORCE_RTOL, (err / scale).max()
