"""ctypes front end of the reference checker (TEST INFRASTRUCTURE ONLY): AdaptiveSph's own kernels run on the CPU
(oracle/ref/ref_host_run.cpp, built into oracle/_ref/ from the reference's sources by oracle/ref/build.py).

It pins the oracle's restatement, and through it the CUDA pipeline, to the reference itself. It exists only where the
reference checkout exists (this build container, not the GPU machine); `available()` says whether it can be used, and
the tests that need it skip otherwise. Only tests/ and the golden-fixture scripts use it.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import OrcParams, OrcRefine, OrcReport, dptr, fptr, make_params, make_refine, uptr  # noqa: F401
from .ref import build as _build

_lib = None
_P = ctypes.POINTER


def available() -> bool:
    try:
        return lib() is not None
    except (OSError, RuntimeError):
        return False


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        if path is None:
            return None
        L = ctypes.CDLL(path)
        f32, u32 = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint32)
        L.ref_boundary_generate.argtypes = [f32, f32, ctypes.c_float, ctypes.c_float, ctypes.c_float, f32, f32,
                                            ctypes.c_uint32]
        L.ref_boundary_generate.restype = ctypes.c_uint32
        L.ref_sim_create.argtypes = [_P(OrcParams), f32, ctypes.c_uint32, f32, f32, ctypes.c_uint32, _P(OrcRefine),
                                     ctypes.c_uint32]
        L.ref_sim_create.restype = ctypes.c_void_p
        L.ref_sim_destroy.argtypes = [ctypes.c_void_p]
        L.ref_sim_step.argtypes = [ctypes.c_void_p, ctypes.c_float]
        L.ref_sim_step.restype = ctypes.c_int
        L.ref_sim_count.argtypes = [ctypes.c_void_p]
        L.ref_sim_count.restype = ctypes.c_uint32
        L.ref_sim_frame.argtypes = [ctypes.c_void_p]
        L.ref_sim_frame.restype = ctypes.c_uint32
        L.ref_set_threads.argtypes = [ctypes.c_int]
        L.ref_sim_read.argtypes = [ctypes.c_void_p] + [f32] * 7 + [u32]
        L.ref_sim_write.argtypes = [ctypes.c_void_p, ctypes.c_uint32] + [f32] * 7 + [u32, ctypes.c_uint32,
                                                                                     ctypes.c_uint32]
        L.ref_sim_density_forces.argtypes = [ctypes.c_void_p]
        L.ref_sim_set_fresh_split_grid.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ref_sim_neighbor_counts.argtypes = [ctypes.c_void_p, u32]
        L.ref_sim_neighbor_counts.restype = ctypes.c_uint64
        L.ref_sim_last_refinement.argtypes = [ctypes.c_void_p, _P(OrcReport)]
        L.ref_sim_last_refinement.restype = ctypes.c_uint32
        _lib = L
    return _lib


def boundary_generate(dmin, dmax, spacing, rho0, h):
    """The reference's StaticBoundaryDomain::generate: (positions (n,4) float32, psi (n,) float32)."""
    L = lib()
    a = (ctypes.c_float * 3)(*dmin)
    b = (ctypes.c_float * 3)(*dmax)
    n = L.ref_boundary_generate(a, b, spacing, rho0, h, None, None, 0)
    pos = np.zeros((max(n, 1), 4), np.float32)
    psi = np.zeros(max(n, 1), np.float32)
    L.ref_boundary_generate(a, b, spacing, rho0, h, fptr(pos), fptr(psi), n)
    return pos[:n].copy(), psi[:n].copy()


class RefSim:
    """The reference's simulation (SphSimulation / AdaptiveSphSimulation) run by its own kernels on the CPU. Arrays
    are in the reference's order (array slots, which its compaction keeps in id order); `id` is the checker's id of
    each particle, numbered as the oracle and the CUDA pipeline number them."""

    def __init__(self, params, positions: np.ndarray, boundary_pos: Optional[np.ndarray] = None,
                 boundary_psi: Optional[np.ndarray] = None, refinement=None, capacity: Optional[int] = None):
        self.L = lib()
        self.P = make_params(params)
        self.R = make_refine(refinement) if refinement is not None and refinement.enabled else None
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
        n = pos.shape[0]
        nb = 0 if boundary_pos is None else int(np.asarray(boundary_pos).reshape(-1, 4).shape[0])
        bp = np.ascontiguousarray(boundary_pos if nb else np.zeros((1, 4)), np.float32).reshape(-1, 4)
        bs = np.ascontiguousarray(boundary_psi if nb else np.zeros(1), np.float32).reshape(-1)
        cap = int(capacity if capacity is not None else n)
        self.cap = max(cap, n, self.R.max_particle_count if self.R is not None else 0, 1)
        self.h = self.L.ref_sim_create(ctypes.byref(self.P), fptr(pos), n, fptr(bp), fptr(bs), nb,
                                       ctypes.byref(self.R) if self.R is not None else None, cap)
        self.report = OrcReport()

    def close(self):
        if self.h:
            self.L.ref_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self) -> int:
        return int(self.L.ref_sim_count(self.h))

    @property
    def frame(self) -> int:
        return int(self.L.ref_sim_frame(self.h))

    def step(self, dt: float) -> bool:
        return bool(self.L.ref_sim_step(self.h, float(dt)))

    def arrays(self) -> dict:
        n = self.n
        out = dict(pos=np.zeros((max(n, 1), 4), np.float32), vel=np.zeros((max(n, 1), 4), np.float32),
                   acc=np.zeros((max(n, 1), 4), np.float32), rho=np.zeros(max(n, 1), np.float32),
                   rad=np.zeros(max(n, 1), np.float32), h=np.zeros(max(n, 1), np.float32),
                   m=np.zeros(max(n, 1), np.float32), id=np.zeros(max(n, 1), np.uint32))
        self.L.ref_sim_read(self.h, *(fptr(out[k]) for k in ("pos", "vel", "acc", "rho", "rad", "h", "m")),
                            uptr(out["id"]))
        return {k: v[:n].copy() for k, v in out.items()}

    def by_id(self) -> dict:
        """arrays() sorted by particle id."""
        a = self.arrays()
        order = np.argsort(a["id"], kind="stable")
        return {k: v[order] for k, v in a.items()}

    def load(self, arrays: dict, frame: int, next_id: int):
        n = int(arrays["pos"].shape[0])
        c = {k: np.ascontiguousarray(arrays[k], np.float32) for k in ("pos", "vel", "acc", "rho", "rad", "h", "m")}
        ids = np.ascontiguousarray(arrays["id"], np.uint32)
        self.L.ref_sim_write(self.h, n, *(fptr(c[k]) for k in ("pos", "vel", "acc", "rho", "rad", "h", "m")),
                             uptr(ids), int(frame), int(next_id))

    def set_fresh_split_grid(self, on: bool = True):
        """Checker option, not the reference's behaviour: rebuild the grid after the merge compaction, before the split
        criterion (the reference walks the step's grid, which the compaction left stale)."""
        self.L.ref_sim_set_fresh_split_grid(self.h, int(bool(on)))

    def density_forces(self):
        """Grid, densities and accelerations of the current positions (no integration)."""
        self.L.ref_sim_density_forces(self.h)

    def neighbor_counts(self) -> np.ndarray:
        out = np.zeros(max(self.n, 1), np.uint32)
        self.L.ref_sim_neighbor_counts(self.h, uptr(out))
        return out[: self.n]

    def last_refinement(self) -> dict:
        bufs = [np.zeros(max(self.cap, 1), np.uint32) for _ in range(3)]
        self.report.removed_ids = uptr(bufs[0])
        self.report.keep_ids = uptr(bufs[1])
        self.report.split_ids = uptr(bufs[2])
        pairs = self.L.ref_sim_last_refinement(self.h, ctypes.byref(self.report))
        d = {k: int(getattr(self.report, k)) for k, _ in OrcReport._fields_[:10]}
        d["removed_ids"] = bufs[0][:pairs].copy()
        d["keep_ids"] = bufs[1][:pairs].copy()
        d["split_ids"] = bufs[2][: d["splits"]].copy()
        return d
