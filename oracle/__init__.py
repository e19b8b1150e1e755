"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the checker for the CUDA pipeline: a CPU restatement of AdaptiveSph's per-step particle pipeline
(see asph_oracle.h for its scope, the reference file:line each function follows, and its parity status:
UNPINNED against the reference's own outputs, which cannot be produced here; pinned by analytic known answers).
Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use it. The product never does.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

from . import build as _build

_lib = None

c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_u32_p = ctypes.POINTER(ctypes.c_uint32)


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("dmin", ctypes.c_float * 3),
        ("dmax", ctypes.c_float * 3),
        ("friction", ctypes.c_float),
        ("gravity", ctypes.c_float * 3),
        ("c0", ctypes.c_float),
        ("rho0", ctypes.c_float),
        ("restitution", ctypes.c_float),
        ("alpha", ctypes.c_float),
        ("sigma", ctypes.c_float),
        ("max_velocity", ctypes.c_float),
        ("h0", ctypes.c_float),
        ("r0", ctypes.c_float),
        ("m0", ctypes.c_float),
        ("threads_per_block", ctypes.c_uint32),
        ("viscosity_model", ctypes.c_uint32),
        ("nu", ctypes.c_float),
        ("periodic", ctypes.c_uint32),
    ]


class OrcRefine(ctypes.Structure):
    _fields_ = [
        ("enabled", ctypes.c_uint32),
        ("min_mass_ratio", ctypes.c_float),
        ("max_mass_ratio", ctypes.c_float),
        ("max_particle_count", ctypes.c_uint32),
        ("max_batch_ratio", ctypes.c_float),
        ("initial_cooldown", ctypes.c_uint32),
        ("cooldown", ctypes.c_uint32),
        ("criterion", ctypes.c_uint32),
        ("eps", ctypes.c_float),
        ("alpha", ctypes.c_float),
        ("center_ratio", ctypes.c_float),
        ("vertex_ratio", ctypes.c_float),
        ("vel_split", ctypes.c_float),
        ("vel_merge", ctypes.c_float),
        ("vort_split", ctypes.c_float),
        ("vort_merge", ctypes.c_float),
        ("curv_split", ctypes.c_float),
        ("curv_merge", ctypes.c_float),
        ("iface_split", ctypes.c_float),
        ("iface_merge", ctypes.c_float),
        ("fs_split", ctypes.c_float),
        ("fs_merge", ctypes.c_float),
    ]


class OrcGrid(ctypes.Structure):
    _fields_ = [
        ("gs", ctypes.c_int32 * 3),
        ("cs", ctypes.c_float * 3),
        ("scale", ctypes.c_float * 3),
        ("dmin", ctypes.c_float * 3),
        ("dmax", ctypes.c_float * 3),
        ("sgs", ctypes.c_int32 * 3),
        ("ncells", ctypes.c_uint32),
        ("bits", ctypes.c_uint32),
        ("periodic", ctypes.c_uint32),
    ]


class OrcState(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint32),
        ("cap", ctypes.c_uint32),
        ("pos", c_float_p),
        ("vel", c_float_p),
        ("acc", c_float_p),
        ("rho", c_float_p),
        ("rad", c_float_p),
        ("h", c_float_p),
        ("m", c_float_p),
        ("id", c_u32_p),
        ("frame", ctypes.c_uint32),
        ("next_id", ctypes.c_uint32),
        ("has_pending", ctypes.c_uint32),
        ("pending_half", ctypes.c_float),
    ]


class OrcState64(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint32),
        ("cap", ctypes.c_uint32),
        ("pos", c_double_p),
        ("vel", c_double_p),
        ("acc", c_double_p),
        ("rho", c_double_p),
        ("rad", c_double_p),
        ("h", c_double_p),
        ("m", c_double_p),
        ("id", c_u32_p),
        ("frame", ctypes.c_uint32),
        ("next_id", ctypes.c_uint32),
        ("has_pending", ctypes.c_uint32),
        ("pending_half", ctypes.c_double),
    ]


class OrcCells(ctypes.Structure):
    _fields_ = [("start", c_u32_p), ("end", c_u32_p), ("keys", c_u32_p), ("ex", ctypes.c_uint32 * 2)]


class OrcBoundary(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint32),
        ("pos", c_float_p),
        ("psi", c_float_p),
        ("fric", c_float_p),
        ("start", c_u32_p),
        ("end", c_u32_p),
        ("ex", ctypes.c_uint32 * 2),
    ]


class OrcReport(ctypes.Structure):
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
        ("capacity_hit", ctypes.c_uint32),
        ("removed_ids", c_u32_p),
        ("keep_ids", c_u32_p),
        ("split_ids", c_u32_p),
    ]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.orc_grid_make.argtypes = [P(OrcParams), P(OrcGrid)]
        L.orc_cell_of.argtypes = [P(OrcGrid), c_float_p, c_u32_p, c_u32_p, c_u32_p]
        L.orc_morton3.argtypes = [ctypes.c_uint32] * 3
        L.orc_morton3.restype = ctypes.c_uint32
        L.orc_sort_stable.argtypes = [ctypes.c_uint32, c_u32_p, ctypes.c_uint32, c_u32_p]
        L.orc_excluded_cells.argtypes = [ctypes.c_uint32, c_u32_p, c_u32_p, c_u32_p]
        L.orc_grid_build.argtypes = [P(OrcGrid), P(OrcState), P(OrcCells)]
        L.orc_cells_from_keys.argtypes = [P(OrcGrid), ctypes.c_uint32, c_u32_p, c_u32_p, c_u32_p]
        L.orc_boundary_setup.argtypes = [P(OrcGrid), ctypes.c_uint32, c_float_p, c_float_p, ctypes.c_float,
                                         P(OrcBoundary)]
        L.orc_boundary_generate.argtypes = [c_float_p, c_float_p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                            c_float_p, c_float_p, ctypes.c_uint32]
        L.orc_boundary_generate.restype = ctypes.c_uint32
        L.orc_cbrtf.argtypes = [ctypes.c_float]
        L.orc_cbrtf.restype = ctypes.c_float
        L.orc32_integrate.argtypes = [P(OrcState), P(OrcParams), ctypes.c_float]
        L.orc32_density.argtypes = [P(OrcGrid), P(OrcParams), P(OrcState), P(OrcCells), P(OrcBoundary), c_float_p]
        L.orc64_density.argtypes = [P(OrcGrid), P(OrcParams), P(OrcState), P(OrcCells), P(OrcBoundary), c_double_p]
        L.orc32_forces.argtypes = [P(OrcGrid), P(OrcParams), P(OrcState), P(OrcCells), P(OrcBoundary), c_float_p]
        L.orc64_forces.argtypes = [P(OrcGrid), P(OrcParams), P(OrcState), P(OrcCells), P(OrcBoundary), c_double_p,
                                   c_double_p]
        L.orc_neighbor_counts.argtypes = [P(OrcGrid), P(OrcState), P(OrcCells), c_u32_p]
        L.orc_list_entries.argtypes = [P(OrcGrid), P(OrcState), P(OrcCells), c_u32_p]
        L.orc_sum_kinds.argtypes = [P(OrcGrid), P(OrcState), P(OrcCells), c_u32_p]
        L.orc32_refine.argtypes = [P(OrcGrid), P(OrcParams), P(OrcRefine), P(OrcState), P(OrcCells), P(OrcReport)]
        L.orc32_step.argtypes = [P(OrcGrid), P(OrcParams), P(OrcRefine), P(OrcState), P(OrcCells), P(OrcBoundary),
                                 ctypes.c_float, P(OrcReport)]
        L.orc32_step.restype = ctypes.c_int
        L.orc_totals.argtypes = [P(OrcParams), P(OrcState), c_double_p]
        L.orc32_export_velocities.argtypes = [P(OrcParams), P(OrcState), c_float_p]
        L.orc64_kernel_w.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc64_kernel_w.restype = ctypes.c_double
        L.orc64_kernel_dw.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc64_kernel_dw.restype = ctypes.c_double
        L.orc32_kernel_w.argtypes = [ctypes.c_float, ctypes.c_float]
        L.orc32_kernel_w.restype = ctypes.c_float
        L.orc_icosahedron.argtypes = [c_float_p]
        L.orc64s_step.argtypes = [P(OrcGrid), P(OrcParams), P(OrcRefine), P(OrcState64), P(OrcCells), P(OrcBoundary),
                                  ctypes.c_double, P(OrcReport)]
        L.orc64s_step.restype = ctypes.c_int
        L.orc64s_totals.argtypes = [P(OrcParams), P(OrcState64), c_double_p]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(c_float_p)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(c_double_p)


def uptr(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(c_u32_p)


def make_params(p) -> OrcParams:
    """OrcParams from adaptivesph_gb300.parameters.Parameters."""
    return OrcParams(
        (ctypes.c_float * 3)(*p.domain.min),
        (ctypes.c_float * 3)(*p.domain.max),
        p.domain.friction,
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


def make_refine(r) -> OrcRefine:
    return OrcRefine(
        int(bool(r.enabled)), r.min_mass_ratio, r.max_mass_ratio, int(r.max_particle_count), r.max_batch_ratio,
        int(r.initial_cooldown), int(r.cooldown), int(r.criterion), r.split_epsilon, r.split_alpha,
        r.split_center_mass_ratio, r.split_vertex_mass_ratio, r.velocity_split_min_speed,
        r.velocity_merge_max_speed, r.vorticity_split_min, r.vorticity_merge_max, r.curvature_split_min,
        r.curvature_merge_max, r.interface_split_distance_ratio, r.interface_merge_distance_ratio,
        r.free_surface_split_deficit, r.free_surface_merge_deficit)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def cbrtf(x: float) -> float:
    return float(lib().orc_cbrtf(float(x)))


def boundary_generate(dmin, dmax, spacing, rho0, h):
    """StaticBoundaryDomain::generate restated: returns (positions (n,4) float32, psi (n,) float32)."""
    L = lib()
    a = (ctypes.c_float * 3)(*dmin)
    b = (ctypes.c_float * 3)(*dmax)
    n = L.orc_boundary_generate(a, b, spacing, rho0, h, None, None, 0)
    pos = np.zeros((max(n, 1), 4), np.float32)
    psi = np.zeros(max(n, 1), np.float32)
    L.orc_boundary_generate(a, b, spacing, rho0, h, fptr(pos), fptr(psi), n)
    return pos[:n].copy(), psi[:n].copy()


class OracleSim:
    """Oracle state in the same internal order as the CUDA pipeline (cell-sorted, splits appended)."""

    def __init__(self, params, positions: np.ndarray, boundary_pos: Optional[np.ndarray] = None,
                 boundary_psi: Optional[np.ndarray] = None, refinement=None, capacity: Optional[int] = None):
        self.L = lib()
        self.params = params
        self.P = make_params(params)
        self.R = make_refine(refinement) if refinement is not None and refinement.enabled else None
        positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
        n = positions.shape[0]
        if capacity is None:
            capacity = refinement.max_particle_count if self.R is not None else n
        cap = max(int(capacity), n, 1)
        self.cap = cap
        self.pos = np.zeros((cap, 4), np.float32)
        self.vel = np.zeros((cap, 4), np.float32)
        self.acc = np.zeros((cap, 4), np.float32)
        self.rho = np.zeros(cap, np.float32)
        self.rad = np.zeros(cap, np.float32)
        self.h = np.zeros(cap, np.float32)
        self.m = np.zeros(cap, np.float32)
        self.id = np.zeros(cap, np.uint32)
        self.pos[:n] = positions
        self.acc[:n, 0:3] = np.asarray(params.gravity, np.float32)
        self.rad[:n] = params.base_particle_radius
        self.h[:n] = params.base_smoothing_radius
        self.m[:n] = params.base_particle_mass
        self.id[:n] = np.arange(n, dtype=np.uint32)
        self.state = OrcState(n, cap, fptr(self.pos), fptr(self.vel), fptr(self.acc), fptr(self.rho), fptr(self.rad),
                              fptr(self.h), fptr(self.m), uptr(self.id), 0, n, 0, 0.0)
        self.grid = OrcGrid()
        self.L.orc_grid_make(ctypes.byref(self.P), ctypes.byref(self.grid))
        nc = self.grid.ncells
        self.cstart = np.full(nc, 0xFFFFFFFF, np.uint32)
        self.cend = np.zeros(nc, np.uint32)
        self.ckeys = np.zeros(cap, np.uint32)
        self.cells = OrcCells(uptr(self.cstart), uptr(self.cend), uptr(self.ckeys), (ctypes.c_uint32 * 2)(0xFFFFFFFF,
                                                                                                          0xFFFFFFFF))
        self.set_boundary(boundary_pos, boundary_psi)
        self.report = OrcReport()
        self._rep_bufs = None

    def set_boundary(self, boundary_pos, boundary_psi):
        nc = self.grid.ncells
        nb = 0 if boundary_pos is None else int(np.asarray(boundary_pos).reshape(-1, 4).shape[0])
        self.bpos = np.zeros((max(nb, 1), 4), np.float32)
        self.bpsi = np.zeros(max(nb, 1), np.float32)
        self.bfric = np.zeros(max(nb, 1), np.float32)
        self.bstart = np.full(nc, 0xFFFFFFFF, np.uint32)
        self.bend = np.zeros(nc, np.uint32)
        self.boundary = OrcBoundary(0, fptr(self.bpos), fptr(self.bpsi), fptr(self.bfric), uptr(self.bstart),
                                    uptr(self.bend), (ctypes.c_uint32 * 2)(0xFFFFFFFF, 0xFFFFFFFF))
        if nb:
            bp = np.ascontiguousarray(boundary_pos, np.float32).reshape(-1, 4)
            bs = np.ascontiguousarray(boundary_psi, np.float32).reshape(-1)
            self.L.orc_boundary_setup(ctypes.byref(self.grid), nb, fptr(bp), fptr(bs), self.params.domain.friction,
                                      ctypes.byref(self.boundary))

    # ------------------------------------------------------------------ state
    @property
    def n(self) -> int:
        return int(self.state.n)

    def arrays(self) -> dict:
        n = self.n
        return dict(pos=self.pos[:n].copy(), vel=self.vel[:n].copy(), acc=self.acc[:n].copy(), rho=self.rho[:n].copy(),
                    rad=self.rad[:n].copy(), h=self.h[:n].copy(), m=self.m[:n].copy(), id=self.id[:n].copy())

    def load(self, arrays: dict, frame: int = 0, next_id: Optional[int] = None, pending_half: Optional[float] = None):
        n = int(arrays["pos"].shape[0])
        assert n <= self.cap
        for k in ("pos", "vel", "acc", "rho", "rad", "h", "m", "id"):
            getattr(self, k)[:n] = arrays[k]
        self.state.n = n
        self.state.frame = frame
        self.state.next_id = int(next_id if next_id is not None else (int(arrays["id"].max()) + 1 if n else 0))
        self.state.has_pending = 0 if pending_half is None else 1
        self.state.pending_half = 0.0 if pending_half is None else float(pending_half)

    # ------------------------------------------------------------------ stages
    def integrate(self, dt: float):
        self.L.orc32_integrate(ctypes.byref(self.state), ctypes.byref(self.P), dt)

    def grid_build(self):
        self.L.orc_grid_build(ctypes.byref(self.grid), ctypes.byref(self.state), ctypes.byref(self.cells))

    def density32(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.float32)
        self.L.orc32_density(ctypes.byref(self.grid), ctypes.byref(self.P), ctypes.byref(self.state),
                             ctypes.byref(self.cells), ctypes.byref(self.boundary), fptr(out))
        return out[: self.n]

    def density64(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.float64)
        self.L.orc64_density(ctypes.byref(self.grid), ctypes.byref(self.P), ctypes.byref(self.state),
                             ctypes.byref(self.cells), ctypes.byref(self.boundary), dptr(out))
        return out[: self.n]

    def forces32(self) -> np.ndarray:
        out = np.zeros((max(self.n, 1), 4), np.float32)
        self.L.orc32_forces(ctypes.byref(self.grid), ctypes.byref(self.P), ctypes.byref(self.state),
                            ctypes.byref(self.cells), ctypes.byref(self.boundary), fptr(out))
        return out[: self.n]

    def forces64(self):
        out = np.zeros((max(self.n, 1), 4), np.float64)
        scale = np.zeros(max(self.n, 1), np.float64)
        self.L.orc64_forces(ctypes.byref(self.grid), ctypes.byref(self.P), ctypes.byref(self.state),
                            ctypes.byref(self.cells), ctypes.byref(self.boundary), dptr(out), dptr(scale))
        return out[: self.n], scale[: self.n]

    def neighbor_counts(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.uint32)
        self.L.orc_neighbor_counts(ctypes.byref(self.grid), ctypes.byref(self.state), ctypes.byref(self.cells),
                                   uptr(out))
        return out[: self.n]

    def list_entries(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.uint32)
        self.L.orc_list_entries(ctypes.byref(self.grid), ctypes.byref(self.state), ctypes.byref(self.cells),
                                uptr(out))
        return out[: self.n]

    def sum_kinds(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.uint32)
        self.L.orc_sum_kinds(ctypes.byref(self.grid), ctypes.byref(self.state), ctypes.byref(self.cells), uptr(out))
        return out[: self.n]

    def _report_buffers(self):
        if self._rep_bufs is None or self._rep_bufs[0].shape[0] < self.cap:
            self._rep_bufs = tuple(np.zeros(self.cap, np.uint32) for _ in range(3))
        self.report.removed_ids = uptr(self._rep_bufs[0])
        self.report.keep_ids = uptr(self._rep_bufs[1])
        self.report.split_ids = uptr(self._rep_bufs[2])

    def refine(self) -> dict:
        assert self.R is not None
        self._report_buffers()
        self.L.orc32_refine(ctypes.byref(self.grid), ctypes.byref(self.P), ctypes.byref(self.R),
                            ctypes.byref(self.state), ctypes.byref(self.cells), ctypes.byref(self.report))
        return self.last_report()

    def last_report(self) -> dict:
        r = self.report
        d = {k: int(getattr(r, k)) for k, _ in OrcReport._fields_[:10]}
        if self._rep_bufs is not None:
            d["removed_ids"] = self._rep_bufs[0][: r.merge_pairs].copy()
            d["keep_ids"] = self._rep_bufs[1][: r.merge_pairs].copy()
            d["split_ids"] = self._rep_bufs[2][: r.splits].copy()
        return d

    def step(self, dt: float) -> bool:
        self._report_buffers()
        refined = self.L.orc32_step(ctypes.byref(self.grid), ctypes.byref(self.P),
                                    ctypes.byref(self.R) if self.R is not None else None, ctypes.byref(self.state),
                                    ctypes.byref(self.cells), ctypes.byref(self.boundary), dt,
                                    ctypes.byref(self.report))
        return bool(refined)

    def totals(self) -> np.ndarray:
        out = np.zeros(6, np.float64)
        self.L.orc_totals(ctypes.byref(self.P), ctypes.byref(self.state), dptr(out))
        return out

    def export_velocities(self) -> np.ndarray:
        out = np.zeros((max(self.n, 1), 4), np.float32)
        self.L.orc32_export_velocities(ctypes.byref(self.P), ctypes.byref(self.state), fptr(out))
        return out[: self.n]

    def sorted_keys(self) -> np.ndarray:
        return self.ckeys[: self.n].copy()

    def excluded(self):
        return int(self.cells.ex[0]), int(self.cells.ex[1])


class OracleSim64(OracleSim):
    """The FP64 step: the same state layout and step as OracleSim, held and advanced in double precision throughout
    (integrate, grid, density, forces, refinement). Created from the same FP32 inputs."""

    def __init__(self, params, positions: np.ndarray, boundary_pos: Optional[np.ndarray] = None,
                 boundary_psi: Optional[np.ndarray] = None, refinement=None, capacity: Optional[int] = None):
        super().__init__(params, positions, boundary_pos, boundary_psi, refinement, capacity)
        n = self.n
        for k in ("pos", "vel", "acc", "rho", "rad", "h", "m"):
            setattr(self, k, getattr(self, k).astype(np.float64))
        self.state = OrcState64(n, self.cap, dptr(self.pos), dptr(self.vel), dptr(self.acc), dptr(self.rho),
                                dptr(self.rad), dptr(self.h), dptr(self.m), uptr(self.id), 0, n, 0, 0.0)

    def load(self, arrays: dict, frame: int = 0, next_id: Optional[int] = None, pending_half: Optional[float] = None):
        super().load({k: np.asarray(v, np.float64) if k != "id" else v for k, v in arrays.items()}, frame, next_id,
                     pending_half)

    def step(self, dt: float) -> bool:
        self._report_buffers()
        refined = self.L.orc64s_step(ctypes.byref(self.grid), ctypes.byref(self.P),
                                     ctypes.byref(self.R) if self.R is not None else None, ctypes.byref(self.state),
                                     ctypes.byref(self.cells), ctypes.byref(self.boundary), float(dt),
                                     ctypes.byref(self.report))
        return bool(refined)

    def totals(self) -> np.ndarray:
        out = np.zeros(6, np.float64)
        self.L.orc64s_totals(ctypes.byref(self.P), ctypes.byref(self.state), dptr(out))
        return out

    def _fp32_only(self, *a, **k):
        raise NotImplementedError("an FP32-state stage; use OracleSim")

    integrate = grid_build = density32 = density64 = forces32 = forces64 = refine = _fp32_only
    neighbor_counts = list_entries = sum_kinds = export_velocities = _fp32_only
