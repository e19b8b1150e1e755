"""The oracle's FP64 step (the CPU step the FP32 pipeline is measured against) against the FP32 oracle, on the CPU:
on a small dam break (plain and adaptive) both keep the same particles and take the same refinement decisions,
densities agree within 1e-5 relative and positions within 1e-6 m after 10-12 steps."""
import numpy as np

import oracle
from helpers import adaptive_refinement, boundary_of, small_dam_break


def _pair(sc):
    bd = boundary_of(sc)
    cap = sc.refinement.max_particle_count if sc.refinement else sc.positions.shape[0]
    args = (sc.parameters, sc.positions, bd.positions, bd.psi, sc.refinement)
    return oracle.OracleSim(*args, capacity=cap), oracle.OracleSim64(*args, capacity=cap)


def test_fp64_step_tracks_fp32_plain():
    sc = small_dam_break()
    o32, o64 = _pair(sc)
    for _ in range(10):
        o32.step(sc.dt)
        o64.step(sc.dt)
    a, b = o32.arrays(), o64.arrays()
    assert b["pos"].dtype == np.float64
    assert np.array_equal(a["id"], b["id"])
    np.testing.assert_allclose(a["rho"], b["rho"], rtol=1e-5)
    np.testing.assert_allclose(a["pos"], b["pos"], atol=1e-6)
    t32, t64 = o32.totals(), o64.totals()
    assert t64[0] == t32[0]  # masses are untouched on a plain step
    assert abs(t64[4] - t32[4]) <= 1e-5 * t64[4]


def test_fp64_step_tracks_fp32_adaptive():
    sc = small_dam_break(refinement=adaptive_refinement())
    o32, o64 = _pair(sc)
    for _ in range(12):
        r32, r64 = o32.step(sc.dt), o64.step(sc.dt)
        assert r32 == r64
    rep32, rep64 = o32.last_report(), o64.last_report()
    assert rep64["merge_pairs"] > 0
    for k in ("count_before", "merge_pairs", "removed", "splits", "count_after"):
        assert rep32[k] == rep64[k], k
    assert o32.n == o64.n
    a, b = o32.arrays(), o64.arrays()
    assert np.array_equal(np.sort(a["id"]), np.sort(b["id"]))
    np.testing.assert_allclose(np.sort(a["m"]), np.sort(b["m"]), rtol=1e-6)
