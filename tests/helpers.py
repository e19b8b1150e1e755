"""Shared builders and comparators for the parity tests (the oracle is the checker)."""
from __future__ import annotations

import numpy as np

import oracle
from adaptivesph_gb300 import StaticBoundaryDomain, create_simulation, scenes
from adaptivesph_gb300.parameters import Criterion, RefinementParameters

STATE_KEYS = ("pos", "vel", "acc", "rho", "rad", "h", "m", "id")


def small_dam_break(counts=(10, 20, 10), dx=0.02, seed=11, tank=(0.6, 0.6, 0.4), refinement=None, walls=True,
                    viscosity=0.01):
    """A small dam break whose walls (0.05 m outside the domain) lie within 2h = 0.052 m of the fluid, so the
    boundary terms are non-zero (with the reference's parameters they vanish, 2h < 0.05 m)."""
    return scenes.dam_break(counts, dx, seed=seed, tank=tank, refinement=refinement, walls=walls,
                            viscosity=viscosity)


def boundary_of(scene):
    if scene.boundary_spacing <= 0:
        return StaticBoundaryDomain.empty(scene.parameters.domain)
    return StaticBoundaryDomain.generate(scene.parameters.domain, scene.boundary_spacing,
                                         scene.parameters.rest_density, scene.parameters.base_smoothing_radius)


def make_pair(scene, capacity=None):
    """(GPU simulation, oracle) created from the same scene."""
    bd = boundary_of(scene)
    cap = capacity if capacity is not None else scene.positions.shape[0]
    sim = create_simulation(scene.parameters, scene.positions, None, None, bd, scene.refinement, cap,
                            max(bd.get_particle_count(), 1))
    orc = oracle.OracleSim(scene.parameters, scene.positions, bd.positions if bd.get_particle_count() else None,
                           bd.psi if bd.get_particle_count() else None, scene.refinement,
                           capacity=scene.refinement.max_particle_count if scene.refinement else cap)
    if scene.velocities is not None:
        st = sim.read_state()
        st["vel"] = scene.velocities.copy()
        sim.write_state(st, next_id=scene.positions.shape[0])
        a = orc.arrays()
        a["vel"] = scene.velocities.copy()
        orc.load(a, next_id=scene.positions.shape[0])
    return sim, orc


def bits(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def assert_bitexact(name, got, want):
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, f"{name}: shape {got.shape} != {want.shape}"
    diff = bits(got) != bits(want)
    if diff.any():
        idx = np.argwhere(diff)[:5]
        raise AssertionError(f"{name}: {int(diff.sum())} entries differ, first at {idx.tolist()}: "
                             f"got {got[tuple(idx[0])]} want {want[tuple(idx[0])]}")


def assert_state_bitexact(gpu_state, orc_state, keys=STATE_KEYS):
    for k in keys:
        assert_bitexact(k, gpu_state[k], orc_state[k])


def adaptive_refinement(criterion=Criterion.VELOCITY, capacity=20000, **kw):
    """Refinement settings that make a small scene merge and split within a few frames."""
    base = dict(enabled=True, min_mass_ratio=0.05, max_mass_ratio=8.0, max_particle_count=capacity,
                max_batch_ratio=0.2, initial_cooldown=2, cooldown=3, criterion=criterion,
                velocity_split_min_speed=0.05, velocity_merge_max_speed=0.2)
    base.update(kw)
    return RefinementParameters(**base)
