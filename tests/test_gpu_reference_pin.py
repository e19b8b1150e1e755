"""The CUDA pipeline against the reference's own results (golden fixtures written by tests/golden/make_ref_golden.py
from AdaptiveSph's kernels run on the CPU; the GPU machine has no reference checkout).

The device rebuilds the fixture's state itself (the same seeded scene and steps, which it computes bit for bit as the
oracle does), then its densities, accelerations, neighbour counts and refinement decisions are compared with the
reference's: integer results equal, densities within 2e-6 relative, accelerations within 1e-5 of the FP64 sum of
|pair terms| + |g| (tolerances and their reasons as in tests/test_reference_pin.py)."""
import os

import numpy as np
import pytest

from adaptivesph_gb300 import scenes
from adaptivesph_gb300.parameters import Criterion
from helpers import adaptive_refinement, make_pair, small_dam_break

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CRITERIA = {
    "velocity": dict(criterion=Criterion.VELOCITY),
    "interface": dict(criterion=Criterion.INTERFACE),
    "vorticity": dict(criterion=Criterion.VORTICITY, vorticity_split_min=2.0, vorticity_merge_max=1.0),
}
REPORT_KEYS = ("frame", "count_before", "merge_eligible", "merge_pairs", "removed", "split_candidates",
               "split_budget", "splits", "count_after")


def _kernels_against_reference(sc, fixture):
    g = np.load(os.path.join(GOLDEN, fixture))
    sim, _ = make_pair(sc)
    for _ in range(int(g["steps"])):
        sim.update(sc.dt)
    st = sim.read_state()
    counts = sim.neighbor_counts()
    order = np.argsort(st["id"], kind="stable")
    pos = np.searchsorted(st["id"][order], g["id"])
    idx = order[pos]
    assert np.array_equal(st["id"][idx], g["id"])
    np.testing.assert_allclose(st["rho"][idx], g["rho"], rtol=2e-6)
    err = np.abs(st["acc"][idx, :3].astype(np.float64) - g["acc"]).max(axis=1)
    worst = float((err / g["scale"]).max())
    assert worst <= 1e-5, worst
    np.testing.assert_array_equal(counts[idx], g["counts"])
    sim.close()


def test_density_forces_counts_match_reference_small_tank():
    _kernels_against_reference(small_dam_break(), "reference_kernels_small_tank.npz")


def test_density_forces_counts_match_reference_128k_sample():
    _kernels_against_reference(scenes.c1_plain(), "reference_kernels_c1_sample.npz")


@pytest.mark.parametrize("name", list(CRITERIA))
def test_refinement_decisions_match_reference(name):
    g = np.load(os.path.join(GOLDEN, "reference_refinement_small.npz"))
    sc = small_dam_break(refinement=adaptive_refinement(**CRITERIA[name]))
    sim, _ = make_pair(sc)
    sim.record_refinement_ids(True)
    reports = g[f"{name}_reports"]
    k = 0
    for _ in range(int(g["frames"])):
        sim.update(sc.dt)
        rep = sim.last_refinement()
        if k < reports.shape[0] and rep["frame"] == reports[k][0] and rep["count_before"] > 0:
            want = dict(zip(REPORT_KEYS, reports[k].tolist()))
            assert {key: rep[key] for key in REPORT_KEYS} == want
            ids = sim.refinement_ids()
            pairs = g[f"{name}_pairs_{k}"]
            assert sorted(ids["keep_ids"].tolist()) == sorted(pairs[:, 0].tolist())
            assert sorted(ids["removed_ids"].tolist()) == sorted(pairs[:, 1].tolist())
            np.testing.assert_array_equal(ids["split_ids"], g[f"{name}_splits_{k}"])
            k += 1
    assert k == reports.shape[0], "every refinement frame of the reference compared"
    assert reports[:, 3].sum() > 0 and reports[:, 7].sum() > 0
    sim.close()
