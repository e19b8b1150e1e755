"""Writes the reference's own results as golden fixtures for the GPU tests (tests/test_gpu_reference_pin.py).

The reference's kernels run on the CPU here (oracle/reference.py, built from the reference's sources; the GPU machine has
no reference checkout), on states produced by the oracle, which the CUDA pipeline reproduces bit for bit. Each
fixture holds the scene's name and the reference's outputs only; the GPU test rebuilds the same state on the device
and compares its own outputs with these.

  reference_kernels_small_tank.npz   small dam break with walls within 2h, after 3 steps: the reference's densities,
                                     accelerations and per-particle neighbour counts on that state, by particle id,
                                     and the FP64 sum of |pair terms| + |g| (force tolerance scale)
  reference_kernels_c1_sample.npz    the plain 128k dam break after 3 steps: the same for every 32nd particle id
  reference_refinement_small.npz     small adaptive dam breaks (velocity, interface, vorticity criterion): the
                                     reference's decisions on each refinement frame of 16 frames (counts, merge
                                     pairs, split parents), taken from the oracle's state before that frame

Run from the repository root: python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from adaptivesph_gb300 import scenes  # noqa: E402
from adaptivesph_gb300.parameters import Criterion  # noqa: E402
from helpers import adaptive_refinement, boundary_of, small_dam_break  # noqa: E402
from oracle import reference  # noqa: E402

REFINE_FRAMES = 16
CRITERIA = {
    "velocity": dict(criterion=Criterion.VELOCITY),
    "interface": dict(criterion=Criterion.INTERFACE),
    "vorticity": dict(criterion=Criterion.VORTICITY, vorticity_split_min=2.0, vorticity_merge_max=1.0),
}


def _pair(sc):
    bd = boundary_of(sc)
    cap = sc.refinement.max_particle_count if sc.refinement else sc.positions.shape[0]
    nb = bd.get_particle_count()
    args = (sc.parameters, sc.positions, bd.positions if nb else None, bd.psi if nb else None, sc.refinement)
    return oracle.OracleSim(*args, capacity=cap), reference.RefSim(*args, capacity=cap)


def kernels(sc, steps, stride):
    o, r = _pair(sc)
    for _ in range(steps):
        o.step(sc.dt)
    st = o.arrays()
    order = np.argsort(st["id"], kind="stable")
    r.load({k: v[order] for k, v in st.items()}, frame=int(o.state.frame), next_id=int(o.state.next_id))
    r.density_forces()
    got = r.by_id()
    counts = r.neighbor_counts()
    o.grid_build()
    _, scale = o.forces64()
    pick = np.arange(0, got["id"].shape[0], stride)
    return dict(steps=np.int32(steps), id=got["id"][pick], rho=got["rho"][pick], acc=got["acc"][pick, :3],
                counts=counts[pick], scale=scale[np.argsort(o.arrays()["id"], kind="stable")][pick])


def refinement(name, kw):
    sc = small_dam_break(refinement=adaptive_refinement(**kw))
    o, r = _pair(sc)
    r.set_fresh_split_grid(True)  # the split criterion on the compacted particles' cells, as this build does
    R = sc.refinement
    rows, pairs, splits = [], [], []
    for f in range(REFINE_FRAMES):
        due = f == R.initial_cooldown or (f > R.initial_cooldown and f % R.cooldown == 0)
        if due:
            st = o.arrays()
            st["vel"] = o.export_velocities()
            order = np.argsort(st["id"], kind="stable")
            r.load({k: v[order] for k, v in st.items()}, frame=int(o.state.frame), next_id=int(o.state.next_id))
        o.step(sc.dt)
        if due:
            r.step(sc.dt)
            rep = r.last_refinement()
            rows.append([rep[k] for k in ("frame", "count_before", "merge_eligible", "merge_pairs", "removed",
                                          "split_candidates", "split_budget", "splits", "count_after")])
            pairs.append(np.stack([rep["keep_ids"], rep["removed_ids"]], axis=1))
            splits.append(rep["split_ids"])
    out = {f"{name}_reports": np.asarray(rows, np.uint32)}
    for k, (p, s) in enumerate(zip(pairs, splits)):
        out[f"{name}_pairs_{k}"] = p.astype(np.uint32)
        out[f"{name}_splits_{k}"] = s.astype(np.uint32)
    return out


def main():
    assert reference.available(), "the reference checkout is needed"
    np.savez_compressed(os.path.join(HERE, "reference_kernels_small_tank.npz"), **kernels(small_dam_break(), 3, 1))
    np.savez_compressed(os.path.join(HERE, "reference_kernels_c1_sample.npz"), **kernels(scenes.c1_plain(), 3, 32))
    out = {"frames": np.int32(REFINE_FRAMES)}
    for name, kw in CRITERIA.items():
        out.update(refinement(name, kw))
    np.savez_compressed(os.path.join(HERE, "reference_refinement_small.npz"), **out)
    for f in sorted(os.listdir(HERE)):
        if f.startswith("reference_"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
