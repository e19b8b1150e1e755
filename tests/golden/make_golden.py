"""Writes the golden fixtures in this folder: the oracle's state after short seeded runs of three small scenes
(plain dam break with walls, adaptive dam break with merges and splits, periodic Taylor-Green with Morris
viscosity). The reference itself cannot be run here (its CUDA library needs glm and nanoflann, which are absent), so
these pin the oracle against later changes of its own code and give the GPU tests a fixed target.

    python tests/golden/make_golden.py          # from the repository root
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from adaptivesph_gb300 import scenes  # noqa: E402
from helpers import adaptive_refinement, boundary_of, small_dam_break  # noqa: E402

KEYS = ("pos", "vel", "rho", "h", "m", "id")


def cases():
    """name -> (scene, steps)"""
    return {
        "plain_dam_break_2k": (small_dam_break(), 20),
        "adaptive_dam_break_2k": (small_dam_break(refinement=adaptive_refinement()), 30),
        "taylor_green_4k": (scenes.taylor_green(16), 12),
    }


def run_oracle(scene, steps):
    """The oracle's state after `steps` steps of `scene` (velocities as stored, export velocities separately)."""
    bd = boundary_of(scene)
    n = scene.positions.shape[0]
    cap = scene.refinement.max_particle_count if scene.refinement else n
    walls = bd.get_particle_count() > 0
    orc = oracle.OracleSim(scene.parameters, scene.positions, bd.positions if walls else None,
                           bd.psi if walls else None, scene.refinement, capacity=cap)
    if scene.velocities is not None:
        a = orc.arrays()
        a["vel"] = scene.velocities.copy()
        orc.load(a, next_id=n)
    for _ in range(steps):
        orc.step(scene.dt)
    out = {k: v.copy() for k, v in orc.arrays().items() if k in KEYS}
    out["export_vel"] = orc.export_velocities().copy()
    return out


def main():
    for name, (scene, steps) in cases().items():
        st = run_oracle(scene, steps)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), steps=np.int32(steps), **st)
        print(name, st["pos"].shape[0], "particles after", steps, "steps")


if __name__ == "__main__":
    main()
