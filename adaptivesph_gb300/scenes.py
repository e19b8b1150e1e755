"""Headless scene generators (the reference's windowed app builds its scene in app/App.cpp:312-341).

All scenes are seeded synthetic data: particle lattices with uniform jitter, the reference's parameter set and
wall boundary. They stand in for the app's JSON-configured scenes (no config file ships with the reference).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional, Tuple

import numpy as np

from .parameters import BoundaryMode, Criterion, Domain, Parameters, RefinementParameters, ViscosityModel

TANK = (1.6, 1.0, 0.67)


@dataclass
class Scene:
    name: str
    parameters: Parameters
    positions: np.ndarray  # (n, 4) float32, w = 0
    refinement: Optional[RefinementParameters]
    dt: float
    velocities: Optional[np.ndarray] = None  # (n, 4) initial velocities, if not at rest
    boundary_spacing: float = 0.0  # 0: no wall particles


def lattice(counts: Tuple[int, int, int], dx: float, origin, jitter: float, seed: int) -> np.ndarray:
    """Particles at origin + (i + 1/2) dx with a uniform jitter of +-jitter*dx per axis."""
    nx, ny, nz = counts
    rng = np.random.default_rng(seed)
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([ii, jj, kk], axis=-1).reshape(-1, 3).astype(np.float64)
    p = (p + 0.5) * dx + np.asarray(origin, np.float64)
    p += rng.uniform(-jitter * dx, jitter * dx, size=p.shape)
    out = np.zeros((p.shape[0], 4), np.float32)
    out[:, :3] = p.astype(np.float32)
    return out


def dam_break(counts=(40, 80, 40), dx: float = 0.01, seed: int = 1, tank=TANK, jitter: float = 0.05,
              h_ratio: float = 1.3, viscosity: float = 0.01, refinement: Optional[RefinementParameters] = None,
              column_height: Optional[float] = None, cfl: float = 0.25, walls: bool = True) -> Scene:
    """Water column in the corner of a closed tank. c0 = 10 sqrt(2 g H), H the column height; h = 1.3 dx;
    m = rho0 dx^3; r0 = dx/2; artificial viscosity alpha (the reference's model); dt = cfl * h / c0."""
    H = column_height if column_height is not None else counts[1] * dx
    c0 = 10.0 * math.sqrt(2.0 * 9.81 * H)
    h = h_ratio * dx
    p = Parameters(
        domain=Domain(min=(0.0, 0.0, 0.0), max=tuple(float(t) for t in tank), friction=0.01),
        gravity=(0.0, -9.81, 0.0),
        speed_of_sound=float(c0),
        rest_density=1000.0,
        restitution=0.5,
        viscosity_constant=viscosity,
        surface_tension_constant=0.0,
        max_velocity=float(10.0 * c0),
        base_smoothing_radius=float(h),
        base_particle_radius=float(dx / 2.0),
        base_particle_mass=float(1000.0 * dx ** 3),
        threads_per_block=256,
    )
    pos = lattice(counts, dx, (0.0, 0.0, 0.0), jitter, seed)
    return Scene("dam_break", p, pos, refinement, float(cfl * h / c0), boundary_spacing=2.0 * p.base_particle_radius
                 if walls else 0.0)


def c1_plain(seed: int = 1) -> Scene:
    """Plain 3D dam break: 40x80x40 = 128,000 particles at dx = 0.01 m."""
    s = dam_break((40, 80, 40), 0.01, seed=seed)
    s.name = "dam_break_plain_128k"
    return s


def c2_refinement(max_particle_count: int = 4_000_000, criterion: Criterion = Criterion.VELOCITY) -> RefinementParameters:
    return RefinementParameters(enabled=True, min_mass_ratio=0.05, max_mass_ratio=8.0,
                                max_particle_count=max_particle_count, max_batch_ratio=0.2, initial_cooldown=10,
                                cooldown=10, criterion=criterion)


def c2_adaptive(seed: int = 2, counts=(100, 200, 50), max_particle_count: int = 4_000_000,
                criterion: Criterion = Criterion.VELOCITY) -> Scene:
    """Adaptive dam break: 100x200x50 = 1,000,000 particles at dx = 0.004 m, velocity criterion (the reference's
    default; Criterion.FREE_SURFACE splits at the free surface instead), minMassRatio 0.05 (two split levels),
    maxMassRatio 8, capacity 4M, batch ratio 0.2, cooldowns 10/10."""
    s = dam_break(counts, 0.004, seed=seed, refinement=c2_refinement(max_particle_count, criterion),
                  column_height=0.8)
    s.name = "dam_break_adaptive_1m"
    return s


def taylor_green(n: int = 128, seed: int = 3, reynolds: float = 100.0, U: float = 1.0, h_ratio: float = 1.3,
                 jitter: float = 0.01) -> Scene:
    """Periodic Taylor-Green vortex in a (2 pi)^3 box: u = U (sin x cos y, -cos x sin y, 0), nu = U L / Re with L = 1,
    Morris viscosity, no gravity, c0 = 10 U."""
    L = 2.0 * math.pi
    dx = L / n
    h = h_ratio * dx
    c0 = 10.0 * U
    nu = U * 1.0 / reynolds
    p = Parameters(
        domain=Domain(min=(0.0, 0.0, 0.0), max=(L, L, L), friction=0.0),
        gravity=(0.0, 0.0, 0.0),
        speed_of_sound=c0,
        rest_density=1000.0,
        restitution=0.0,
        viscosity_constant=0.0,
        surface_tension_constant=0.0,
        max_velocity=100.0 * U,
        base_smoothing_radius=h,
        base_particle_radius=dx / 2.0,
        base_particle_mass=1000.0 * dx ** 3,
        threads_per_block=256,
        viscosity_model=ViscosityModel.MORRIS,
        kinematic_viscosity=nu,
        boundary_mode=BoundaryMode.PERIODIC,
    )
    pos = lattice((n, n, n), dx, (0.0, 0.0, 0.0), jitter, seed)
    x, y = pos[:, 0].astype(np.float64), pos[:, 1].astype(np.float64)
    vel = np.zeros_like(pos)
    vel[:, 0] = (U * np.sin(x) * np.cos(y)).astype(np.float32)
    vel[:, 1] = (-U * np.cos(x) * np.sin(y)).astype(np.float32)
    return Scene("taylor_green", p, pos, None, float(0.25 * h / (c0 + U)), velocities=vel)


def batched_mix(count: int = 256, seed: int = 4, dx: float = 0.01, min_particles: int = 4096,
                max_particles: int = 262144):
    """Independent dam-break scenes of uneven sizes for batched stepping: particle counts log-uniform in
    [min_particles, max_particles], fill fraction U(0.2, 0.6), Morris viscosity nu log-uniform in [1e-6, 1e-3],
    refinement (velocity criterion, two split levels) on the even-numbered scenes. Each fluid block is
    nx x 2nx x nx particles at spacing dx in the corner of a tank 1.25 times the block's height and as deep as the
    block, whose length makes the fluid fill the requested fraction of the tank."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n_target = math.exp(rng.uniform(math.log(min_particles), math.log(max_particles)))
        fill = rng.uniform(0.2, 0.6)
        nu = math.exp(rng.uniform(math.log(1e-6), math.log(1e-3)))
        nx = max(4, int(round((n_target / 2.0) ** (1.0 / 3.0))))
        height = 2 * nx * dx
        tank = (0.8 * nx * dx / fill, 1.25 * height, nx * dx)
        refinement = None
        if k % 2 == 0:
            refinement = RefinementParameters(enabled=True, min_mass_ratio=0.05, max_mass_ratio=8.0,
                                              max_particle_count=2 * (2 * nx ** 3), max_batch_ratio=0.2,
                                              initial_cooldown=10, cooldown=10, criterion=Criterion.VELOCITY)
        s = dam_break((nx, 2 * nx, nx), dx, seed=seed * 1000 + k, tank=tank, refinement=refinement)
        s.parameters.viscosity_model = ViscosityModel.MORRIS
        s.parameters.kinematic_viscosity = float(nu)
        s.name = f"mix_{k:03d}"
        out.append(s)
    return out


def served_requests(count: int = 24, seed: int = 5, min_particles: int = 8192, max_particles: int = 1_000_000,
                    refinement_probability: float = 0.5, min_steps: int = 200, max_steps: int = 2000):
    """Scene requests for the serving loop: dam breaks whose spacing gives a particle count log-uniform in
    [min_particles, max_particles] (nx x 2nx x nx lattice in a 1.6 x 1.0 x 0.67 m tank, the column 0.8 m high),
    refinement (velocity criterion, two split levels) with the given probability, a step count uniform in
    [min_steps, max_steps]. Returns (scene, steps) pairs in arrival order."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n_target = math.exp(rng.uniform(math.log(min_particles), math.log(max_particles)))
        nx = max(8, int(round((n_target / 2.0) ** (1.0 / 3.0))))
        dx = 0.4 / nx  # the column is 0.4 m wide and 0.8 m high, whatever the resolution
        refine = rng.uniform() < refinement_probability
        steps = int(rng.integers(min_steps, max_steps + 1))
        refinement = None
        if refine:
            refinement = RefinementParameters(enabled=True, min_mass_ratio=0.05, max_mass_ratio=8.0,
                                              max_particle_count=2 * (2 * nx ** 3), max_batch_ratio=0.2,
                                              initial_cooldown=10, cooldown=10, criterion=Criterion.VELOCITY)
        s = dam_break((nx, 2 * nx, nx), dx, seed=seed * 1000 + k, refinement=refinement, column_height=0.8)
        s.name = f"request_{k:03d}"
        out.append((s, steps))
    return out
