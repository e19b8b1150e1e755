"""The free-surface refinement criterion (neighbour-count deficit; no reference counterpart) in the oracle, on the
CPU: the split parents it picks on a resting fluid block lie at the block's free faces, never at the faces that touch
the domain, and its FP32 (canonical, what the CUDA kernels compute) and FP64 decisions agree over 30 frames."""
import numpy as np

import oracle
from adaptivesph_gb300.parameters import Criterion
from helpers import adaptive_refinement, boundary_of, small_dam_break


def _pair(sc, fp64=False):
    bd = boundary_of(sc)
    cls = oracle.OracleSim64 if fp64 else oracle.OracleSim
    return cls(sc.parameters, sc.positions, bd.positions, bd.psi, sc.refinement,
               capacity=sc.refinement.max_particle_count)


def test_split_parents_are_at_the_free_faces():
    """A 10 x 20 x 10 block at dx = 0.02 in the corner of the tank, refined at frame 0 (before it moves): merges in
    the bulk free particles, and the split parents are then the particles with the largest deficit, which must lie
    within 2h of the block's free faces (x, y, z at the block's far side) and at least 2h from every domain face."""
    R = adaptive_refinement(criterion=Criterion.FREE_SURFACE, initial_cooldown=0, cooldown=10)
    sc = small_dam_break(refinement=R)
    o = _pair(sc)
    pos0 = {int(i): p for i, p in zip(o.arrays()["id"], o.arrays()["pos"])}
    assert o.step(sc.dt)
    rep = o.last_report()
    assert rep["merge_pairs"] > 0 and rep["splits"] > 0
    h = sc.parameters.base_smoothing_radius
    block_max = sc.positions[:, :3].max(axis=0)
    dmin = np.array(sc.parameters.domain.min)
    dmax = np.array(sc.parameters.domain.max)
    for i in rep["split_ids"].tolist():
        p = pos0[i][:3]
        assert (block_max - p).min() < 2 * h, (i, p)                  # at a free face
        assert min((p - dmin).min(), (dmax - p).min()) >= 2 * h - 1e-4  # not at a domain face


def test_fp32_and_fp64_decisions_agree():
    sc = small_dam_break(refinement=adaptive_refinement(criterion=Criterion.FREE_SURFACE))
    o32, o64 = _pair(sc), _pair(sc, fp64=True)
    splits = 0
    for _ in range(30):
        assert o32.step(sc.dt) == o64.step(sc.dt)
        a, b = o32.last_report(), o64.last_report()
        for k in ("merge_eligible", "merge_pairs", "split_candidates", "split_budget", "splits", "count_after"):
            assert a[k] == b[k], k
        splits += a["splits"]
    assert splits > 0
