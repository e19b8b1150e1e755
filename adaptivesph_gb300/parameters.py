"""Parameter types mirroring the reference's simulation interface, and their C-ABI layouts.

Python mirrors of ``sph::cuda::Simulation::Parameters`` (cuda/include/cuda/simulation/Simulation.cuh:64-109),
``Simulation::Parameters::Domain`` (:66-94), ``refinement::RefinementParameters`` and its nested structs
(cuda/include/cuda/refinement/RefinementParameters.cuh:6-104), ``Simulation::DensityInfo`` (Simulation.cuh:111-120)
and ``physics::StaticBoundaryDomain::Particle`` (StaticBoundaryDomain.cuh:17-21). The ctypes structures match
include/asph.h field for field. Defaults are the reference's defaults.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass, field
from typing import Tuple

Vec3 = Tuple[float, float, float]


class Criterion(enum.IntEnum):
    """RefinementParameters::Criterion (RefinementParameters.cuh:82-87)."""

    VELOCITY = 0
    INTERFACE = 1
    VORTICITY = 2
    FREE_SURFACE = 3  # neighbour-count deficit; no reference counterpart


class ViscosityModel(enum.IntEnum):
    ARTIFICIAL = 0  # the reference's Monaghan-type viscosity (Algorithm.cu:110-174)
    MORRIS = 1  # Morris, Fox & Zhu (1997); no reference counterpart


class BoundaryMode(enum.IntEnum):
    CLAMP = 0  # the reference's clamp to the domain box (Algorithm.cu:286-298)
    PERIODIC = 1  # periodic box; no reference counterpart


@dataclass
class Domain:
    """Simulation::Parameters::Domain (Simulation.cuh:66-94)."""

    min: Vec3 = (-1.0, -1.0, -1.0)
    max: Vec3 = (1.0, 1.0, 1.0)
    friction: float = 0.01

    def get_translation(self) -> Vec3:
        return tuple((a + b) / 2.0 for a, b in zip(self.max, self.min))  # type: ignore[return-value]

    def get_scale(self) -> Vec3:
        return tuple(a - b for a, b in zip(self.max, self.min))  # type: ignore[return-value]

    def get_volume(self) -> float:
        s = self.get_scale()
        return s[0] * s[1] * s[2]

    @staticmethod
    def from_transform(translation: Vec3, scale: Vec3) -> "Domain":
        return Domain(
            min=tuple(t - s / 2.0 for t, s in zip(translation, scale)),  # type: ignore[arg-type]
            max=tuple(t + s / 2.0 for t, s in zip(translation, scale)),  # type: ignore[arg-type]
        )


@dataclass
class Parameters:
    """Simulation::Parameters (Simulation.cuh:64-109) plus three extensions (viscosity model, Morris nu,
    boundary mode). The reference has no defaults for the physical fields."""

    domain: Domain = field(default_factory=Domain)
    gravity: Vec3 = (0.0, -9.81, 0.0)
    speed_of_sound: float = 10.0
    rest_density: float = 1000.0
    restitution: float = 0.5
    viscosity_constant: float = 0.01
    surface_tension_constant: float = 0.0
    max_velocity: float = 100.0
    base_smoothing_radius: float = 0.013
    base_particle_radius: float = 0.005
    base_particle_mass: float = 0.001
    threads_per_block: int = 256
    viscosity_model: ViscosityModel = ViscosityModel.ARTIFICIAL
    kinematic_viscosity: float = 0.0
    boundary_mode: BoundaryMode = BoundaryMode.CLAMP


@dataclass
class RefinementParameters:
    """refinement::RefinementParameters (RefinementParameters.cuh:80-104) with the nested Splitting, Velocity,
    Vorticity, Curvature and Interface parameters flattened; defaults as in the reference."""

    enabled: bool = False
    min_mass_ratio: float = 0.3
    max_mass_ratio: float = 8.0
    max_particle_count: int = 1_000_000
    max_batch_ratio: float = 0.2
    initial_cooldown: int = 10
    cooldown: int = 10
    criterion: Criterion = Criterion.VELOCITY
    split_epsilon: float = 0.65
    split_alpha: float = 0.70
    split_center_mass_ratio: float = 0.077
    split_vertex_mass_ratio: float = 0.077
    velocity_split_min_speed: float = 2.0
    velocity_merge_max_speed: float = 0.1
    vorticity_split_min: float = 1.0
    vorticity_merge_max: float = 0.3
    curvature_split_min: float = 2.0
    curvature_merge_max: float = 0.6
    interface_split_distance_ratio: float = 0.05
    interface_merge_distance_ratio: float = 0.15
    # extension: the free-surface criterion's neighbour-count deficits (split at or above, merge at or below)
    free_surface_split_deficit: float = 0.25
    free_surface_merge_deficit: float = 0.05


@dataclass
class DensityInfo:
    """Simulation::DensityInfo (Simulation.cuh:111-120)."""

    rest_density: float
    min_density: float
    max_density: float
    average_density: float
    under_density_count: int
    normal_density_count: int
    over_density_count: int


# ----------------------------------------------------------------------------------------------- C layouts
class CDomain(ctypes.Structure):
    _fields_ = [("min", ctypes.c_float * 3), ("max", ctypes.c_float * 3), ("friction", ctypes.c_float)]


class CParameters(ctypes.Structure):
    _fields_ = [
        ("domain", CDomain),
        ("gravity", ctypes.c_float * 3),
        ("speed_of_sound", ctypes.c_float),
        ("rest_density", ctypes.c_float),
        ("restitution", ctypes.c_float),
        ("viscosity_constant", ctypes.c_float),
        ("surface_tension_constant", ctypes.c_float),
        ("max_velocity", ctypes.c_float),
        ("base_smoothing_radius", ctypes.c_float),
        ("base_particle_radius", ctypes.c_float),
        ("base_particle_mass", ctypes.c_float),
        ("threads_per_block", ctypes.c_uint32),
        ("viscosity_model", ctypes.c_uint32),
        ("kinematic_viscosity", ctypes.c_float),
        ("boundary_mode", ctypes.c_uint32),
    ]


class CRefinementParameters(ctypes.Structure):
    _fields_ = [
        ("enabled", ctypes.c_uint32),
        ("min_mass_ratio", ctypes.c_float),
        ("max_mass_ratio", ctypes.c_float),
        ("max_particle_count", ctypes.c_uint32),
        ("max_batch_ratio", ctypes.c_float),
        ("initial_cooldown", ctypes.c_uint32),
        ("cooldown", ctypes.c_uint32),
        ("criterion", ctypes.c_uint32),
        ("split_epsilon", ctypes.c_float),
        ("split_alpha", ctypes.c_float),
        ("split_center_mass_ratio", ctypes.c_float),
        ("split_vertex_mass_ratio", ctypes.c_float),
        ("velocity_split_min_speed", ctypes.c_float),
        ("velocity_merge_max_speed", ctypes.c_float),
        ("vorticity_split_min", ctypes.c_float),
        ("vorticity_merge_max", ctypes.c_float),
        ("curvature_split_min", ctypes.c_float),
        ("curvature_merge_max", ctypes.c_float),
        ("interface_split_distance_ratio", ctypes.c_float),
        ("interface_merge_distance_ratio", ctypes.c_float),
        ("free_surface_split_deficit", ctypes.c_float),
        ("free_surface_merge_deficit", ctypes.c_float),
    ]


class CBoundaryParticle(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 4), ("psi", ctypes.c_float)]


class CDensityInfo(ctypes.Structure):
    _fields_ = [
        ("rest_density", ctypes.c_float),
        ("min_density", ctypes.c_float),
        ("max_density", ctypes.c_float),
        ("average_density", ctypes.c_float),
        ("under_density_count", ctypes.c_uint32),
        ("normal_density_count", ctypes.c_uint32),
        ("over_density_count", ctypes.c_uint32),
    ]


class CTotals(ctypes.Structure):
    _fields_ = [
        ("mass", ctypes.c_double),
        ("momentum", ctypes.c_double * 3),
        ("kinetic_energy", ctypes.c_double),
        ("volume", ctypes.c_double),
        ("count", ctypes.c_uint32),
    ]


class CStateInfo(ctypes.Structure):
    _fields_ = [
        ("count", ctypes.c_uint32),
        ("capacity", ctypes.c_uint32),
        ("frame", ctypes.c_uint32),
        ("next_id", ctypes.c_uint32),
        ("pending_half_dt", ctypes.c_float),
        ("has_pending", ctypes.c_uint32),
    ]


class CGridInfo(ctypes.Structure):
    _fields_ = [
        ("reference_cells", ctypes.c_int32 * 3),
        ("reference_cell_size", ctypes.c_float * 3),
        ("sub_cells", ctypes.c_int32 * 3),
        ("cell_count", ctypes.c_uint32),
        ("key_bits", ctypes.c_uint32),
        ("excluded_cells", ctypes.c_uint32 * 2),
        ("boundary_excluded_cells", ctypes.c_uint32 * 2),
    ]


class CRefinementReport(ctypes.Structure):
    _fields_ = [
        ("frame", ctypes.c_uint32),
        ("count_before", ctypes.c_uint32),
        ("merge_eligible", ctypes.c_uint32),
        ("merge_pairs", ctypes.c_uint32),
        ("removed", ctypes.c_uint32),
        ("split_candidates", ctypes.c_uint32),
        ("split_budget", ctypes.c_uint32),
        ("splits", ctypes.c_uint32),
        ("count_after", ctypes.c_uint32),
    ]


class CRequest(ctypes.Structure):
    _fields_ = [
        ("parameters", CParameters),
        ("positions", ctypes.POINTER(ctypes.c_float)),
        ("count", ctypes.c_uint32),
        ("boundary", ctypes.POINTER(CBoundaryParticle)),
        ("boundary_count", ctypes.c_uint32),
        ("refinement", ctypes.POINTER(CRefinementParameters)),
        ("max_fluid_capacity", ctypes.c_uint32),
        ("delta_time", ctypes.c_float),
        ("steps", ctypes.c_uint32),
        ("wall_spacing", ctypes.c_float),
    ]


class CRequestStatus(ctypes.Structure):
    _fields_ = [
        ("state", ctypes.c_uint32),
        ("steps_done", ctypes.c_uint32),
        ("steps", ctypes.c_uint32),
        ("count", ctypes.c_uint32),
        ("error", ctypes.c_int),
        ("device_bytes", ctypes.c_uint64),
        ("submit_s", ctypes.c_double),
        ("admit_s", ctypes.c_double),
        ("finish_s", ctypes.c_double),
    ]


def to_c_domain(d: Domain) -> CDomain:
    return CDomain((ctypes.c_float * 3)(*d.min), (ctypes.c_float * 3)(*d.max), d.friction)


def to_c_parameters(p: Parameters) -> CParameters:
    return CParameters(
        to_c_domain(p.domain),
        (ctypes.c_float * 3)(*p.gravity),
        p.speed_of_sound,
        p.rest_density,
        p.restitution,
        p.viscosity_constant,
        p.surface_tension_constant,
        p.max_velocity,
        p.base_smoothing_radius,
        p.base_particle_radius,
        p.base_particle_mass,
        int(p.threads_per_block),
        int(p.viscosity_model),
        p.kinematic_viscosity,
        int(p.boundary_mode),
    )


def to_c_refinement(r: RefinementParameters) -> CRefinementParameters:
    return CRefinementParameters(
        int(bool(r.enabled)),
        r.min_mass_ratio,
        r.max_mass_ratio,
        int(r.max_particle_count),
        r.max_batch_ratio,
        int(r.initial_cooldown),
        int(r.cooldown),
        int(r.criterion),
        r.split_epsilon,
        r.split_alpha,
        r.split_center_mass_ratio,
        r.split_vertex_mass_ratio,
        r.velocity_split_min_speed,
        r.velocity_merge_max_speed,
        r.vorticity_split_min,
        r.vorticity_merge_max,
        r.curvature_split_min,
        r.curvature_merge_max,
        r.interface_split_distance_ratio,
        r.interface_merge_distance_ratio,
        r.free_surface_split_deficit,
        r.free_surface_merge_deficit,
    )
