"""Python mirror of the reference's simulation interface over the C ABI.

``create_simulation`` / ``Simulation`` follow ``sph::cuda::createSimulation`` and the ``Simulation`` virtuals
(cuda/include/cuda/simulation/Simulation.cuh:61-145); ``StaticBoundaryDomain.generate`` follows
StaticBoundaryDomain.cuh:23-26; ``import_buffer`` / ``ImportedMemory`` follow ImportedMemory.cuh:10-26. Names keep
the reference's meaning, argument order and defaults; failures raise ``AsphError`` (the C ABI returns a status
where the reference returns nothing).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from . import parameters as _p
from .parameters import DensityInfo, Domain, Parameters, RefinementParameters

_vp = ctypes.c_void_p


def _fp(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _up(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


class ImportedMemory:
    """A device buffer the simulation writes into (ImportedMemory.cuh:10-20)."""

    def __init__(self, handle: int):
        self._h = _vp(handle)

    @property
    def handle(self):
        return self._h

    def device_pointer(self) -> int:
        out = _vp()
        _lib.check(_lib.load().asph_memory_device_pointer(self._h, ctypes.byref(out)), "asph_memory_device_pointer")
        return int(out.value or 0)

    def size(self) -> int:
        out = ctypes.c_size_t()
        _lib.check(_lib.load().asph_memory_size(self._h, ctypes.byref(out)), "asph_memory_size")
        return int(out.value)

    def release(self) -> None:
        if self._h:
            _lib.load().asph_memory_release(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def import_buffer(handle: int, size: int) -> ImportedMemory:
    """importBuffer(int handle, size_t size) (ImportedMemory.cuh:25): imports a Vulkan opaque FD."""
    out = _vp()
    _lib.check(_lib.load().asph_import_buffer_fd(int(handle), int(size), ctypes.byref(out)), "importBuffer")
    return ImportedMemory(out.value)


def allocate_buffer(size: int) -> ImportedMemory:
    """Headless stand-in for an imported buffer: a device allocation of ``size`` bytes."""
    out = _vp()
    _lib.check(_lib.load().asph_memory_allocate(int(size), ctypes.byref(out)), "asph_memory_allocate")
    return ImportedMemory(out.value)


@dataclass
class FluidParticlesDataImportedBuffer:
    """Simulation.cuh:46-52"""

    positions: ImportedMemory
    velocities: ImportedMemory
    densities: ImportedMemory
    radii: ImportedMemory


@dataclass
class BoundaryParticlesDataImportedBuffer:
    """Simulation.cuh:54-59"""

    positions: ImportedMemory
    radii: ImportedMemory
    colors: ImportedMemory


class StaticBoundaryDomain:
    """physics::StaticBoundaryDomain (StaticBoundaryDomain.cuh:14-50). Like the reference's domain, which holds its
    particles as one array of BoundaryParticle records that createSimulation copies as they are, it keeps the
    records (asph_boundary_particle: x, y, z, w, psi) built once, so creating a simulation passes them without a
    conversion (3-6 ms for the 503,100 walls of the 1M dam break). positions and psi are read-only copies."""

    def __init__(self, bounds: Domain, positions: np.ndarray, psi: np.ndarray, _records=None):
        self.bounds = bounds
        self.positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
        self.psi = np.ascontiguousarray(psi, np.float32).reshape(-1)
        n = self.positions.shape[0]
        if self.psi.shape[0] != n:
            raise ValueError("one psi per boundary particle")
        if _records is None:
            _records = (_p.CBoundaryParticle * max(n, 1))()
            if n:
                raw = np.frombuffer(_records, dtype=np.float32).reshape(-1, 5)
                raw[:n, :4] = self.positions
                raw[:n, 4] = self.psi
        self._records = _records
        self.positions.setflags(write=False)
        self.psi.setflags(write=False)

    @staticmethod
    def generate(bounds: Domain, particle_spacing: float, fluid_rest_density: float,
                 fluid_smoothing_radius: float, device: bool = False) -> "StaticBoundaryDomain":
        """StaticBoundaryDomain::generate; device=True runs it on the GPU (asph_boundary_generate_gpu, bit-identical
        output)."""
        lib = _lib.load()
        fn = lib.asph_boundary_generate_gpu if device else lib.asph_boundary_generate
        d = _p.to_c_domain(bounds)
        n = ctypes.c_uint32()
        _lib.check(fn(ctypes.byref(d), particle_spacing, fluid_rest_density, fluid_smoothing_radius, None, 0,
                      ctypes.byref(n)), "StaticBoundaryDomain::generate")
        arr = (_p.CBoundaryParticle * max(n.value, 1))()
        _lib.check(fn(ctypes.byref(d), particle_spacing, fluid_rest_density, fluid_smoothing_radius,
                      ctypes.cast(arr, _vp), n.value, ctypes.byref(n)), "StaticBoundaryDomain::generate")
        raw = np.frombuffer(arr, dtype=np.float32).reshape(-1, 5)[: n.value]
        return StaticBoundaryDomain(bounds, raw[:, :4].copy(), raw[:, 4].copy(), _records=arr)

    @staticmethod
    def empty(bounds: Domain) -> "StaticBoundaryDomain":
        return StaticBoundaryDomain(bounds, np.zeros((0, 4), np.float32), np.zeros(0, np.float32))

    def get_particle_count(self) -> int:
        return int(self.positions.shape[0])

    def to_c(self):
        return self._records, self.get_particle_count()


class Simulation:
    """sph::cuda::Simulation (Simulation.cuh:61-136) over the C ABI."""

    def __init__(self, handle, parameters: Parameters, refinement: Optional[RefinementParameters]):
        self._h = _vp(handle)
        self._lib = _lib.load()
        self.parameters = parameters
        self.refinement = refinement

    # -------------------------------------------------------------------- reference interface
    def update(self, delta_time: float) -> None:
        """Simulation::update (SphSimulation.cu:101-120): one step, returns after the device is done."""
        _lib.check(self._lib.asph_simulation_update(self._h, float(delta_time)), "update")

    def update_domain(self, domain: Domain, boundary_domain: StaticBoundaryDomain) -> None:
        arr, n = boundary_domain.to_c()
        d = _p.to_c_domain(domain)
        _lib.check(self._lib.asph_simulation_update_domain(self._h, ctypes.byref(d), ctypes.cast(arr, _vp), n),
                   "updateDomain")
        self.parameters.domain = domain

    def get_fluid_particles_count(self) -> int:
        out = ctypes.c_uint32()
        _lib.check(self._lib.asph_simulation_fluid_count(self._h, ctypes.byref(out)), "getFluidParticlesCount")
        return int(out.value)

    def device_bytes(self) -> int:
        out = ctypes.c_uint64()
        _lib.check(self._lib.asph_simulation_device_bytes(self._h, ctypes.byref(out)), "device_bytes")
        return int(out.value)

    def get_boundary_particles_count(self) -> int:
        out = ctypes.c_uint32()
        _lib.check(self._lib.asph_simulation_boundary_count(self._h, ctypes.byref(out)), "getBoundaryParticlesCount")
        return int(out.value)

    def calculate_average_neighbor_count(self) -> float:
        out = ctypes.c_float()
        _lib.check(self._lib.asph_simulation_average_neighbor_count(self._h, ctypes.byref(out)),
                   "calculateAverageNeighborCount")
        return float(out.value)

    def get_density_info(self, threshold: float) -> DensityInfo:
        out = _p.CDensityInfo()
        _lib.check(self._lib.asph_simulation_density_info(self._h, float(threshold), ctypes.byref(out)),
                   "getDensityInfo")
        return DensityInfo(out.rest_density, out.min_density, out.max_density, out.average_density,
                           out.under_density_count, out.normal_density_count, out.over_density_count)

    def enable_adaptive_refinement(self) -> None:
        _lib.check(self._lib.asph_simulation_enable_adaptive_refinement(self._h), "enableAdaptiveRefinement")

    # -------------------------------------------------------------------- extensions
    def step_async(self, delta_time: float) -> None:
        _lib.check(self._lib.asph_simulation_step_async(self._h, float(delta_time)), "step_async")

    def step_cfl(self, cfl: float = 0.25, dt_max: float = 0.0) -> float:
        dt = ctypes.c_float()
        _lib.check(self._lib.asph_simulation_step_cfl(self._h, cfl, dt_max, ctypes.byref(dt)), "step_cfl")
        return float(dt.value)

    def synchronize(self) -> None:
        _lib.check(self._lib.asph_simulation_synchronize(self._h), "synchronize")

    def run_stages(self, delta_time: float, last_stage: int) -> None:
        _lib.check(self._lib.asph_simulation_run_stages(self._h, float(delta_time), int(last_stage)), "run_stages")

    def export(self) -> None:
        _lib.check(self._lib.asph_simulation_export(self._h), "export")

    def export_host(self, out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        n = self.get_fluid_particles_count()
        if out is None:
            out = dict(positions=np.zeros((n, 4), np.float32), velocities=np.zeros((n, 4), np.float32),
                       densities=np.zeros(n, np.float32), radii=np.zeros(n, np.float32), ids=np.zeros(n, np.uint32))
        cap = min(v.shape[0] for v in out.values()) if out else 0
        _lib.check(self._lib.asph_simulation_export_host(self._h, _fp(out.get("positions")),
                                                         _fp(out.get("velocities")), _fp(out.get("densities")),
                                                         _fp(out.get("radii")), _up(out.get("ids")), cap),
                   "export_host")
        return out

    def export_host_async(self, out: Dict[str, np.ndarray]) -> Dict[str, np.ndarray]:
        """Enqueues the export into `out` (pinned arrays for asynchronous copies) and returns at once; the arrays
        hold the particles of this point of the stream after export_wait()."""
        cap = min(v.shape[0] for v in out.values()) if out else 0
        _lib.check(self._lib.asph_simulation_export_host_async(self._h, _fp(out.get("positions")),
                                                               _fp(out.get("velocities")), _fp(out.get("densities")),
                                                               _fp(out.get("radii")), _up(out.get("ids")), cap),
                   "export_host_async")
        return out

    def export_wait(self) -> None:
        _lib.check(self._lib.asph_simulation_export_wait(self._h), "export_wait")

    def totals(self) -> Dict[str, float]:
        t = _p.CTotals()
        _lib.check(self._lib.asph_simulation_totals(self._h, ctypes.byref(t)), "totals")
        return dict(mass=t.mass, momentum=(t.momentum[0], t.momentum[1], t.momentum[2]),
                    kinetic_energy=t.kinetic_energy, volume=t.volume, count=t.count)

    def device_errors(self, clear: bool = False) -> int:
        out = ctypes.c_uint32()
        _lib.check(self._lib.asph_simulation_device_errors(self._h, ctypes.byref(out), int(clear)), "device_errors")
        return int(out.value)

    def set_stream(self, stream: int) -> None:
        _lib.check(self._lib.asph_simulation_set_stream(self._h, _vp(stream) if stream else None), "set_stream")

    def state_info(self) -> Dict[str, float]:
        s = _p.CStateInfo()
        _lib.check(self._lib.asph_simulation_state_info(self._h, ctypes.byref(s)), "state_info")
        return dict(count=s.count, capacity=s.capacity, frame=s.frame, next_id=s.next_id,
                    pending_half_dt=s.pending_half_dt, has_pending=bool(s.has_pending))

    def read_state(self) -> Dict[str, np.ndarray]:
        n = self.get_fluid_particles_count()
        out = dict(pos=np.zeros((n, 4), np.float32), vel=np.zeros((n, 4), np.float32), acc=np.zeros((n, 4), np.float32),
                   rho=np.zeros(n, np.float32), rad=np.zeros(n, np.float32), h=np.zeros(n, np.float32),
                   m=np.zeros(n, np.float32), id=np.zeros(n, np.uint32))
        _lib.check(self._lib.asph_simulation_read_fluid(self._h, _fp(out["pos"]), _fp(out["vel"]), _fp(out["acc"]),
                                                        _fp(out["rho"]), _fp(out["rad"]), _fp(out["h"]), _fp(out["m"]),
                                                        _up(out["id"]), n), "read_fluid")
        return out

    def write_state(self, state: Dict[str, np.ndarray], frame: int = 0, next_id: Optional[int] = None,
                    pending_half: Optional[float] = None) -> None:
        n = int(state["pos"].shape[0])
        info = _p.CStateInfo(n, 0, int(frame),
                             int(next_id if next_id is not None else (int(state["id"].max()) + 1 if n else 0)),
                             float(pending_half or 0.0), 0 if pending_half is None else 1)
        c = {k: np.ascontiguousarray(state[k], np.uint32 if k == "id" else np.float32)
             for k in ("pos", "vel", "acc", "rho", "rad", "h", "m", "id")}
        _lib.check(self._lib.asph_simulation_write_fluid(self._h, ctypes.byref(info), _fp(c["pos"]), _fp(c["vel"]),
                                                         _fp(c["acc"]), _fp(c["rho"]), _fp(c["rad"]), _fp(c["h"]),
                                                         _fp(c["m"]), _up(c["id"])), "write_fluid")

    def grid_info(self) -> Dict[str, object]:
        g = _p.CGridInfo()
        _lib.check(self._lib.asph_simulation_grid_info(self._h, ctypes.byref(g)), "grid_info")
        return dict(reference_cells=tuple(g.reference_cells), reference_cell_size=tuple(g.reference_cell_size),
                    sub_cells=tuple(g.sub_cells), cell_count=g.cell_count, key_bits=g.key_bits,
                    excluded_cells=tuple(g.excluded_cells), boundary_excluded_cells=tuple(g.boundary_excluded_cells))

    def read_grid(self) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = self.get_fluid_particles_count()
        nc = int(self.grid_info()["cell_count"])
        keys = np.zeros(max(n, 1), np.uint32)
        start = np.zeros(nc, np.uint32)
        end = np.zeros(nc, np.uint32)
        _lib.check(self._lib.asph_simulation_read_grid(self._h, _up(keys), keys.shape[0], _up(start), _up(end), nc),
                   "read_grid")
        return keys[:n], start, end

    def neighbor_counts(self) -> np.ndarray:
        n = self.get_fluid_particles_count()
        out = np.zeros(max(n, 1), np.uint32)
        _lib.check(self._lib.asph_simulation_neighbor_counts(self._h, _up(out), out.shape[0]), "neighbor_counts")
        return out[:n]

    def last_refinement(self) -> Dict[str, int]:
        r = _p.CRefinementReport()
        _lib.check(self._lib.asph_simulation_last_refinement(self._h, ctypes.byref(r)), "last_refinement")
        return {k: int(getattr(r, k)) for k, _ in _p.CRefinementReport._fields_}

    def record_refinement_ids(self, enable: bool = True) -> None:
        _lib.check(self._lib.asph_debug_record_refinement(self._h, int(enable)), "record_refinement")

    def refinement_ids(self) -> Dict[str, np.ndarray]:
        rep = self.last_refinement()
        cap = max(rep["merge_pairs"], rep["splits"], 1)
        keep = np.zeros(cap, np.uint32)
        rem = np.zeros(cap, np.uint32)
        spl = np.zeros(cap, np.uint32)
        _lib.check(self._lib.asph_debug_refinement_ids(self._h, _up(keep), _up(rem), _up(spl), cap), "refinement_ids")
        return dict(keep_ids=keep[: rep["merge_pairs"]], removed_ids=rem[: rep["merge_pairs"]],
                    split_ids=spl[: rep["splits"]])

    def enable_timing(self, enable: bool = True) -> None:
        _lib.check(self._lib.asph_simulation_enable_timing(self._h, int(enable)), "enable_timing")

    def kernel_times(self) -> Dict[str, Tuple[float, int]]:
        n = len(_lib.KERNEL_CLASSES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_uint32 * n)()
        _lib.check(self._lib.asph_simulation_kernel_times(self._h, ms, cnt, n), "kernel_times")
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(_lib.KERNEL_CLASSES)}

    def launch_count(self) -> int:
        out = ctypes.c_uint64()
        _lib.check(self._lib.asph_simulation_launch_count(self._h, ctypes.byref(out)), "launch_count")
        return int(out.value)

    def close(self) -> None:
        if self._h:
            self._lib.asph_simulation_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def create_simulation(parameters: Parameters, positions: np.ndarray,
                      fluid_particle_memory: Optional[FluidParticlesDataImportedBuffer],
                      boundary_particle_memory: Optional[BoundaryParticlesDataImportedBuffer],
                      boundary_domain: StaticBoundaryDomain, refinement_params: Optional[RefinementParameters],
                      max_fluid_particle_capacity: int, max_boundary_particle_capacity: int) -> Simulation:
    """sph::cuda::createSimulation (Simulation.cuh:138-145, SimulationFactory.cu:14-40): adaptive when
    refinement_params is given and enabled, plain otherwise."""
    lib = _lib.load()
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
    cp = _p.to_c_parameters(parameters)
    cr = _p.to_c_refinement(refinement_params) if refinement_params is not None else None
    fb = None
    if fluid_particle_memory is not None:
        f = fluid_particle_memory
        fb = (ctypes.c_void_p * 4)(f.positions.handle, f.velocities.handle, f.densities.handle, f.radii.handle)
    bb = None
    if boundary_particle_memory is not None:
        b = boundary_particle_memory
        bb = (ctypes.c_void_p * 3)(b.positions.handle, b.radii.handle, b.colors.handle)
    arr, nb = boundary_domain.to_c()
    out = _vp()
    _lib.check(lib.asph_simulation_create(ctypes.byref(cp), _fp(pos), pos.shape[0],
                                          ctypes.cast(fb, _vp) if fb is not None else None,
                                          ctypes.cast(bb, _vp) if bb is not None else None,
                                          ctypes.cast(arr, _vp), nb, ctypes.byref(cr) if cr is not None else None,
                                          int(max_fluid_particle_capacity), int(max_boundary_particle_capacity),
                                          ctypes.byref(out)), "createSimulation")
    sim = Simulation(out.value, parameters, refinement_params)
    sim._keepalive = (fluid_particle_memory, boundary_particle_memory)
    return sim


def create_simulation_with_walls(parameters: Parameters, positions: np.ndarray, wall_spacing: float,
                                 refinement_params: Optional[RefinementParameters], max_fluid_particle_capacity: int,
                                 max_boundary_particle_capacity: int = 0) -> Simulation:
    """StaticBoundaryDomain::generate on the GPU followed by createSimulation (asph_simulation_create_with_walls):
    the walls never pass through host memory and equal those of StaticBoundaryDomain.generate bit for bit."""
    lib = _lib.load()
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
    cp = _p.to_c_parameters(parameters)
    cr = _p.to_c_refinement(refinement_params) if refinement_params is not None else None
    out = _vp()
    _lib.check(lib.asph_simulation_create_with_walls(ctypes.byref(cp), _fp(pos), pos.shape[0], None, None,
                                                     float(wall_spacing), ctypes.byref(cr) if cr is not None else None,
                                                     int(max_fluid_particle_capacity),
                                                     int(max_boundary_particle_capacity), ctypes.byref(out)),
               "createSimulation (walls on the device)")
    return Simulation(out.value, parameters, refinement_params)


class _TuningInfo(ctypes.Structure):
    """asph_batch_tuning_info (include/asph.h)."""

    _fields_ = [("mode", ctypes.c_uint32), ("tuned", ctypes.c_uint32), ("segmented", ctypes.c_uint32 * 3),
                ("chunk", ctypes.c_uint32), ("ctas_per_sm", ctypes.c_uint32), ("trials", ctypes.c_uint32),
                ("segmented_steps", ctypes.c_uint64), ("segmented_captures", ctypes.c_uint64),
                ("trial_ms", ctypes.c_double * 16), ("trial_config", ctypes.c_uint32 * 16)]


BATCH_MODES = {"auto": 0, "graphs": 1, "segmented": 2}


class Batch:
    """Independent simulations advanced together (asph_batch_*; no reference counterpart): their steps overlap on
    the device. Plain frames run as per-simulation graphs or through segmented density and force passes shared by
    up to 64 simulations (mode "graphs", "segmented", or "auto": an autotuner picks per particle-count bucket). Each
    simulation's result equals its result when stepped alone, in every mode. The batch does not own the
    simulations; keep them alive while the batch exists."""

    def __init__(self, simulations: Sequence[Simulation], mode: str = "auto"):
        self._lib = _lib.load()
        self._sims = list(simulations)
        arr = (_vp * max(len(self._sims), 1))(*[s._h.value for s in self._sims])
        h = _vp()
        _lib.check(self._lib.asph_batch_create(arr, len(self._sims), ctypes.byref(h)), "asph_batch_create")
        self._h = h
        self.set_mode(mode)

    def set_mode(self, mode: str) -> None:
        _lib.check(self._lib.asph_batch_set_mode(self._h, BATCH_MODES[mode]), "asph_batch_set_mode")

    def tuning(self) -> Dict[str, object]:
        t = _TuningInfo()
        _lib.check(self._lib.asph_batch_tuning(self._h, ctypes.byref(t)), "asph_batch_tuning")
        names = {v: k for k, v in BATCH_MODES.items()}
        trials = []
        for q in range(t.trials):
            c = t.trial_config[q]
            trials.append(dict(segmented=[(c >> b) & 1 for b in range(3)], chunk=(c >> 8) & 0xFF,
                               ctas_per_sm=(c >> 16) & 0xFF, ms_per_frame=float(t.trial_ms[q])))
        return dict(mode=names.get(t.mode, t.mode), tuned=bool(t.tuned), segmented=list(t.segmented),
                    chunk=t.chunk, ctas_per_sm=t.ctas_per_sm, segmented_steps=t.segmented_steps,
                    segmented_captures=t.segmented_captures, trials=trials,
                    buckets="particle counts below 16384, below 65536, and above")

    def step(self, delta_times, steps: int = 1) -> None:
        dts = np.ascontiguousarray(np.broadcast_to(np.asarray(delta_times, np.float32), (len(self._sims),)))
        _lib.check(self._lib.asph_batch_step(self._h, _fp(dts), int(steps)), "asph_batch_step")

    def stats(self) -> Dict[str, int]:
        g, e, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(self._lib.asph_batch_stats(self._h, ctypes.byref(g), ctypes.byref(e), ctypes.byref(c)),
                   "asph_batch_stats")
        return dict(graph_steps=g.value, eager_steps=e.value, captures=c.value)

    def close(self) -> None:
        if self._h:
            self._lib.asph_batch_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_device_bytes(parameters: Parameters, count: int, boundary_count: int,
                          refinement: Optional[RefinementParameters], max_fluid_capacity: int) -> int:
    """Device memory asph_simulation_create would allocate for these arguments."""
    lib = _lib.load()
    cp = _p.to_c_parameters(parameters)
    cr = _p.to_c_refinement(refinement) if refinement is not None and refinement.enabled else None
    out = ctypes.c_uint64()
    _lib.check(lib.asph_estimate_device_bytes(ctypes.byref(cp), int(count), int(boundary_count),
                                              ctypes.byref(cr) if cr is not None else None, int(max_fluid_capacity),
                                              int(boundary_count), ctypes.byref(out)), "estimate_device_bytes")
    return int(out.value)


REQUEST_STATES = {0: "queued", 1: "active", 2: "done", 3: "failed"}


class Server:
    """The serving loop (asph_server_*; no reference counterpart): requests queue, are admitted first come first
    served under a device-memory budget, run together, and retire with their particles copied to host memory."""

    def __init__(self, memory_budget_bytes: int, max_active: int = 0):
        self._lib = _lib.load()
        h = _vp()
        _lib.check(self._lib.asph_server_create(int(memory_budget_bytes), int(max_active), ctypes.byref(h)),
                   "asph_server_create")
        self._h = h

    def submit(self, parameters: Parameters, positions: np.ndarray, boundary: Optional["StaticBoundaryDomain"],
               refinement: Optional[RefinementParameters], delta_time: float, steps: int,
               max_fluid_capacity: Optional[int] = None, wall_spacing: float = 0.0) -> int:
        """boundary None with wall_spacing > 0: the walls are generated on the GPU at admission."""
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
        bp, nb = boundary.to_c() if boundary is not None else (None, 0)
        cr = _p.to_c_refinement(refinement) if refinement is not None and refinement.enabled else None
        cap = max_fluid_capacity if max_fluid_capacity is not None else pos.shape[0]
        rq = _p.CRequest(_p.to_c_parameters(parameters), _fp(pos), pos.shape[0],
                         ctypes.cast(bp, ctypes.POINTER(_p.CBoundaryParticle)) if nb else None,
                         nb, ctypes.pointer(cr) if cr is not None else None, int(cap),
                         float(delta_time), int(steps), float(wall_spacing))
        t = ctypes.c_uint64()
        _lib.check(self._lib.asph_server_submit(self._h, ctypes.byref(rq), ctypes.byref(t)), "asph_server_submit")
        return int(t.value)

    def poll(self, max_steps: int = 0) -> int:
        out = ctypes.c_uint32()
        _lib.check(self._lib.asph_server_poll(self._h, int(max_steps), ctypes.byref(out)), "asph_server_poll")
        return int(out.value)

    def status(self, ticket: int) -> Dict[str, object]:
        s = _p.CRequestStatus()
        _lib.check(self._lib.asph_server_status(self._h, int(ticket), ctypes.byref(s)), "asph_server_status")
        return dict(state=REQUEST_STATES.get(s.state, "?"), steps_done=s.steps_done, steps=s.steps, count=s.count,
                    error=s.error, device_bytes=s.device_bytes, submit_s=s.submit_s, admit_s=s.admit_s,
                    finish_s=s.finish_s)

    def take(self, ticket: int) -> Dict[str, np.ndarray]:
        n = int(self.status(ticket)["count"])
        out = dict(positions=np.zeros((n, 4), np.float32), velocities=np.zeros((n, 4), np.float32),
                   densities=np.zeros(n, np.float32), radii=np.zeros(n, np.float32), ids=np.zeros(n, np.uint32))
        _lib.check(self._lib.asph_server_take(self._h, int(ticket), _fp(out["positions"]), _fp(out["velocities"]),
                                              _fp(out["densities"]), _fp(out["radii"]), _up(out["ids"]), n),
                   "asph_server_take")
        return out

    def stats(self) -> Dict[str, int]:
        used, q, a = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
        g, e = ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(self._lib.asph_server_stats(self._h, ctypes.byref(used), ctypes.byref(q), ctypes.byref(a),
                                               ctypes.byref(g), ctypes.byref(e)), "asph_server_stats")
        return dict(used_bytes=used.value, queued=q.value, active=a.value, graph_steps=g.value, eager_steps=e.value)

    def close(self) -> None:
        if self._h:
            self._lib.asph_server_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
