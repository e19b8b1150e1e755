"""AdaptiveSph's own CUDA kernels on the GPU (TEST AND MEASUREMENT INFRASTRUCTURE ONLY): the reference's plain step
(SphSimulation::update, cuda/src/simulation/SphSimulation.cu:101-120) run with the reference's kernels, compiled
from its sources for sm_103a by oracle/ref/build.py (oracle/_ref/ref_*.cubin) and launched here through the CUDA
driver API. It is the reference arm's GPU leg (bench.py --impl reference) and is checked against the reference's
CPU-run results by tests/test_gpu_reference_cuda.py; the product never loads it.

What is the reference's and what is restated:
* every kernel is the reference's, compiled unchanged with the reference's CUDA options, launched with the
  reference's block size (Parameters::threadsPerBlock) and grid (ceil(count / threadsPerBlock)), in the order of
  SphSimulation::update, on one stream, with a device synchronisation at the end of every step as the reference
  does;
* the host orchestration is restated (SphSimulation.cu:28-80 constructor state, :101-120 update, :179-235 the
  launches; NeighborGrid.cu:33-150 grid size, tables and update), because those files are host C++ that runs
  beside the kernels;
* NeighborGrid::resetGrid's thrust::fill_n of -1 (NeighborGrid.cu:129-133) is a device fill of the same bytes, and
  NeighborGrid::sortParticles's thrust::sort_by_key of the int32 cell indices (NeighborGrid.cu:134-140; Thrust's
  radix sort of integer keys is stable) is torch.sort(stable=True) of the same keys, whose permutation is the
  sorted particleArrayIndices because assignParticlesToCells writes particleArrayIndices[i] = i: both are CUB radix
  sorts;
* kernel arguments are packed from the byte layout that oracle/ref/ref_layout_probe.cpp recorded from the
  reference's headers (oracle/_ref/ref_layout.json), and every argument's size is checked against the kernel's own
  parameter table (cuFuncGetParamInfo) before the first launch.
The reference's refinement pass (AdaptiveSphSimulation) is not run here: its compaction moves particles in place
while other threads read them (the race the CPU checker orders away), so only the plain step is timed on the GPU.
"""
from __future__ import annotations

import ctypes
import json
import os
import re
import struct
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
MODULES = ("algorithm", "boundary", "neighbors")
LAYOUT = os.path.join(OUT, "ref_layout.json")

# kernel -> (module, argument kinds in order); the signatures are Algorithm.cuh:12-28, BoundaryAlgorithm.cuh,
# NeighborKernels.cuh:9-10
KERNELS = {
    "computeDensities": ("algorithm", ("fluid", "device")),
    "computePressureAccelerations": ("algorithm", ("fluid", "device", "params")),
    "computeViscosityAccelerations": ("algorithm", ("fluid", "device", "params")),
    "computeSurfaceTensionAccelerations": ("algorithm", ("fluid", "device", "params")),
    "computeExternalAccelerations": ("algorithm", ("fluid", "params")),
    "halfKickVelocities": ("algorithm", ("fluid", "params", "f32")),
    "updatePositions": ("algorithm", ("fluid", "domain", "f32")),
    "sumAllNeighbors": ("algorithm", ("fluid", "device", "ptr")),
    "computeBoundaryDensityContribution": ("boundary", ("fluid", "boundary", "device")),
    "computeBoundaryPressureAcceleration": ("boundary", ("fluid", "boundary", "device", "params")),
    "computeBoundaryFrictionAcceleration": ("boundary", ("fluid", "boundary", "device", "params")),
    "assignParticlesToCells": ("neighbors", ("ptr", "device", "griddata")),
    "calculateCellStartAndEndIndices": ("neighbors", ("griddata",)),
}


def cubin(name: str) -> str:
    return os.path.join(OUT, f"ref_{name}.cubin")


def available() -> bool:
    """True where the reference's cubins and their argument layout exist and a GPU is present."""
    if not all(os.path.exists(cubin(m)) for m in MODULES) or not os.path.exists(LAYOUT):
        return False
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


class _Driver:
    """The few CUDA driver API entry points the launcher needs (libcuda, through ctypes)."""

    def __init__(self):
        cu = ctypes.CDLL("libcuda.so.1")
        P, vp, sz = ctypes.POINTER, ctypes.c_void_p, ctypes.c_size_t
        cu.cuInit.argtypes = [ctypes.c_uint]
        cu.cuCtxGetCurrent.argtypes = [P(vp)]
        cu.cuModuleLoad.argtypes = [P(vp), ctypes.c_char_p]
        cu.cuModuleUnload.argtypes = [vp]
        cu.cuModuleGetFunctionCount.argtypes = [P(ctypes.c_uint), vp]
        cu.cuModuleEnumerateFunctions.argtypes = [P(vp), ctypes.c_uint, vp]
        cu.cuFuncGetName.argtypes = [P(ctypes.c_char_p), vp]
        cu.cuFuncGetParamInfo.argtypes = [vp, sz, P(sz), P(sz)]
        cu.cuLaunchKernel.argtypes = [vp, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                      ctypes.c_uint, ctypes.c_uint, vp, P(vp), P(vp)]
        cu.cuGetErrorString.argtypes = [ctypes.c_int, P(ctypes.c_char_p)]
        for f in ("cuInit", "cuCtxGetCurrent", "cuModuleLoad", "cuModuleUnload", "cuModuleGetFunctionCount",
                  "cuModuleEnumerateFunctions", "cuFuncGetName", "cuFuncGetParamInfo", "cuLaunchKernel",
                  "cuGetErrorString"):
            getattr(cu, f).restype = ctypes.c_int
        self.cu = cu
        self.check(cu.cuInit(0), "cuInit")

    def check(self, r: int, what: str):
        if r != 0:
            s = ctypes.c_char_p()
            self.cu.cuGetErrorString(r, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {r} ({(s.value or b'?').decode()})")


def _kernel_name(mangled: str) -> Optional[str]:
    """The unqualified name of a kernel in namespace sph::cuda::kernel, from its Itanium-mangled name."""
    m = re.match(r"_ZN3sph4cuda6kernel(\d+)", mangled)
    if not m:
        return None
    k = int(m.group(1))
    start = m.end()
    return mangled[start:start + k]


class RefCudaSim:
    """The reference's plain simulation (SphSimulation) on the GPU, run by its own kernels. Arrays live in torch
    device tensors; particles keep their slots (the reference never reorders particle data)."""

    def __init__(self, params, positions: np.ndarray, boundary_pos: Optional[np.ndarray] = None,
                 boundary_psi: Optional[np.ndarray] = None, capacity: Optional[int] = None):
        import torch

        self.torch = torch
        torch.cuda.init()
        self.dev = torch.device("cuda", torch.cuda.current_device())
        torch.zeros(1, device=self.dev)  # the runtime's primary context is current from here on
        self.drv = _Driver()
        ctx = ctypes.c_void_p()
        self.drv.check(self.drv.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        with open(LAYOUT) as f:
            self.layout = json.load(f)
        self._load_kernels()

        p = params
        f32 = np.float32
        self.P = p
        self.tpb = int(p.threads_per_block)
        pos = np.ascontiguousarray(positions, f32).reshape(-1, 4)
        self.n = int(pos.shape[0])
        self.cap = int(max(capacity or self.n, self.n, 1))
        self.nb = 0 if boundary_pos is None else int(np.asarray(boundary_pos).reshape(-1, 4).shape[0])
        T = lambda shape, dt=torch.float32: torch.zeros(shape, dtype=dt, device=self.dev)  # noqa: E731
        # SphSimulation constructor state (SphSimulation.cu:28-80): velocities 0, accelerations = (gravity, 0),
        # radii r0, smoothing radii h0, masses m0
        self.pos = T((self.cap, 4))
        self.pos[:self.n] = torch.from_numpy(pos).to(self.dev)
        self.vel = T((self.cap, 4))
        self.acc = T((self.cap, 4))
        self.acc[:, :3] = torch.tensor([float(f32(g)) for g in p.gravity], dtype=torch.float32, device=self.dev)
        self.rho = T(self.cap)
        self.rad = torch.full((self.cap,), f32(p.base_particle_radius), device=self.dev)
        self.h = torch.full((self.cap,), f32(p.base_smoothing_radius), device=self.dev)
        self.m = torch.full((self.cap,), f32(p.base_particle_mass), device=self.dev)
        nb1 = max(self.nb, 1)
        self.bpos = T((nb1, 4))
        self.bpsi = T(nb1)
        if self.nb:
            self.bpos[:self.nb] = torch.from_numpy(np.ascontiguousarray(boundary_pos, f32).reshape(-1, 4)).to(self.dev)
            self.bpsi[:self.nb] = torch.from_numpy(np.ascontiguousarray(boundary_psi, f32).reshape(-1)).to(self.dev)
        # initializeBoundaryParticles (SphSimulation.cu:287-333): colours, friction coefficients, radii
        self.bcol = torch.tensor([0.3, 0.3, 0.3, 0.2], dtype=torch.float32, device=self.dev).repeat(nb1, 1)
        self.bvisc = torch.full((nb1,), f32(p.domain.friction), device=self.dev)
        self.brad = torch.full((nb1,), f32(p.base_particle_radius), device=self.dev)
        # NeighborGrid::createGrid (NeighborGrid.cu:103-121) with the cell width of SphSimulation.cu:47, in float
        dmin = np.array(p.domain.min, f32)
        dmax = np.array(p.domain.max, f32)
        scale = (dmax - dmin).astype(f32)
        width = f32(f32(2.0) * f32(p.base_smoothing_radius)) * f32(self.layout["wendlandRangeRatio"])
        self.grid_size = np.ceil((scale / width).astype(f32)).astype(np.int32)
        self.cell_size = (scale / self.grid_size.astype(f32)).astype(f32)
        cells = int(np.prod(self.grid_size.astype(np.int64)))
        I32 = torch.int32
        self.f_start, self.f_end = T(cells, I32), T(cells, I32)
        self.f_gidx, self.f_aidx = T(self.cap, I32), T(self.cap, I32)
        self.b_start, self.b_end = T(cells, I32), T(cells, I32)
        self.b_gidx, self.b_aidx = T(nb1, I32), T(nb1, I32)
        self.cells = cells
        self.count_buf = T(1, I32)
        self.stream = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        if self.nb:
            self._update_grid(boundary=True)  # SphSimulation.cu:77-79
        torch.cuda.synchronize()

    # ------------------------------------------------------------------ kernels and their arguments
    def _load_kernels(self):
        cu = self.drv.cu
        self.modules = {}
        names: Dict[str, ctypes.c_void_p] = {}
        for m in MODULES:
            mod = ctypes.c_void_p()
            self.drv.check(cu.cuModuleLoad(ctypes.byref(mod), cubin(m).encode()), f"cuModuleLoad({m})")
            self.modules[m] = mod
            cnt = ctypes.c_uint()
            self.drv.check(cu.cuModuleGetFunctionCount(ctypes.byref(cnt), mod), "cuModuleGetFunctionCount")
            funcs = (ctypes.c_void_p * cnt.value)()
            self.drv.check(cu.cuModuleEnumerateFunctions(funcs, cnt.value, mod), "cuModuleEnumerateFunctions")
            for fn in funcs:
                nm = ctypes.c_char_p()
                self.drv.check(cu.cuFuncGetName(ctypes.byref(nm), fn), "cuFuncGetName")
                k = _kernel_name(nm.value.decode())
                if k in KERNELS and KERNELS[k][0] == m:
                    names[k] = ctypes.c_void_p(fn)
        missing = sorted(set(KERNELS) - set(names))
        if missing:
            raise RuntimeError(f"reference kernels not found in the cubins: {missing}")
        self.funcs = names
        sizes = {"fluid": self.layout["FluidParticlesData"]["size"], "device": self.layout["Device"]["size"],
                 "params": self.layout["Parameters"]["size"], "boundary": self.layout["BoundaryParticlesData"]["size"],
                 "domain": self.layout["Domain"]["size"], "griddata": self.layout["GridData"]["size"],
                 "f32": 4, "ptr": 8}
        # every argument's size against the kernel's own parameter table; no launch happens on a mismatch
        for k, (_, kinds) in KERNELS.items():
            for idx, kind in enumerate(kinds):
                off, size = ctypes.c_size_t(), ctypes.c_size_t()
                self.drv.check(cu.cuFuncGetParamInfo(names[k], idx, ctypes.byref(off), ctypes.byref(size)),
                               f"cuFuncGetParamInfo({k}, {idx})")
                if size.value != sizes[kind]:
                    raise RuntimeError(f"{k} argument {idx}: {size.value} bytes in the kernel, {sizes[kind]} packed")
            off, size = ctypes.c_size_t(), ctypes.c_size_t()
            if cu.cuFuncGetParamInfo(names[k], len(kinds), ctypes.byref(off), ctypes.byref(size)) == 0:
                raise RuntimeError(f"{k} takes more arguments than packed")

    @staticmethod
    def _put(buf: bytearray, off: int, fmt: str, *vals):
        struct.pack_into("<" + fmt, buf, off, *vals)

    def _fluid(self) -> bytes:
        L = self.layout["FluidParticlesData"]
        b = bytearray(L["size"])
        for f, t in (("positions", self.pos), ("velocities", self.vel), ("accelerations", self.acc),
                     ("densities", self.rho), ("radii", self.rad), ("smoothingRadii", self.h), ("masses", self.m)):
            self._put(b, L[f], "Q", t.data_ptr())
        self._put(b, L["particleCount"], "I", self.n)
        return bytes(b)

    def _boundary(self) -> bytes:
        L = self.layout["BoundaryParticlesData"]
        b = bytearray(L["size"])
        for f, t in (("positions", self.bpos), ("colors", self.bcol), ("psiValues", self.bpsi),
                     ("viscosityCoefficients", self.bvisc), ("radii", self.brad)):
            self._put(b, L[f], "Q", t.data_ptr())
        self._put(b, L["particleCount"], "I", self.nb)
        return bytes(b)

    def _domain_into(self, b: bytearray, base: int):
        L = self.layout["Domain"]
        d = self.P.domain
        self._put(b, base + L["min"], "3f", *d.min)
        self._put(b, base + L["max"], "3f", *d.max)
        self._put(b, base + L["friction"], "f", d.friction)

    def _domain(self) -> bytes:
        b = bytearray(self.layout["Domain"]["size"])
        self._domain_into(b, 0)
        return bytes(b)

    def _params(self) -> bytes:
        L = self.layout["Parameters"]
        p = self.P
        b = bytearray(L["size"])
        self._domain_into(b, L["domain"])
        self._put(b, L["gravity"], "3f", *p.gravity)
        for f, v in (("speedOfSound", p.speed_of_sound), ("restDensity", p.rest_density),
                     ("restitution", p.restitution), ("viscosityConstant", p.viscosity_constant),
                     ("surfaceTensionConstant", p.surface_tension_constant), ("maxVelocity", p.max_velocity),
                     ("baseSmoothingRadius", p.base_smoothing_radius), ("baseParticleRadius", p.base_particle_radius),
                     ("baseParticleMass", p.base_particle_mass)):
            self._put(b, L[f], "f", v)
        self._put(b, L["threadsPerBlock"], "I", self.tpb)
        return bytes(b)

    def _griddata_into(self, b: bytearray, base: int, boundary: bool):
        L = self.layout["GridData"]
        start, end, gidx, aidx = ((self.b_start, self.b_end, self.b_gidx, self.b_aidx) if boundary
                                  else (self.f_start, self.f_end, self.f_gidx, self.f_aidx))
        for f, t in (("cellStartIndices", start), ("cellEndIndices", end), ("particleGridIndices", gidx),
                     ("particleArrayIndices", aidx)):
            self._put(b, base + L[f + ".data"], "Q", t.data_ptr())
            self._put(b, base + L[f + ".size"], "Q", t.numel())
        self._put(b, base + L["particleCount"], "I", self.nb if boundary else self.n)

    def _griddata(self, boundary: bool) -> bytes:
        b = bytearray(self.layout["GridData"]["size"])
        self._griddata_into(b, 0, boundary)
        return bytes(b)

    def _device(self) -> bytes:
        L = self.layout["Device"]
        G = self.layout["Grid"]
        b = bytearray(L["size"])
        self._domain_into(b, L["domain"])
        self._put(b, L["grid"] + G["gridSize"], "3i", *(int(v) for v in self.grid_size))
        self._put(b, L["grid"] + G["cellSize"], "3f", *(float(v) for v in self.cell_size))
        self._griddata_into(b, L["fluid"], False)
        self._griddata_into(b, L["boundary"], True)
        return bytes(b)

    def _launch(self, name: str, count: int, *args: bytes):
        if count == 0:
            return
        bufs = [ctypes.create_string_buffer(a, len(a)) for a in args]
        ptrs = (ctypes.c_void_p * len(bufs))(*[ctypes.cast(x, ctypes.c_void_p) for x in bufs])
        blocks = (count + self.tpb - 1) // self.tpb
        self.drv.check(self.drv.cu.cuLaunchKernel(self.funcs[name], blocks, 1, 1, self.tpb, 1, 1, 0, self.stream,
                                                  ptrs, None), f"cuLaunchKernel({name})")

    # ------------------------------------------------------------------ the reference's step
    def _update_grid(self, boundary: bool):
        """NeighborGrid::updateFluid / updateBoundary (NeighborGrid.cu:33-50): reset the tables, assign cells, sort
        by cell, start/end indices."""
        start, end, gidx, aidx = ((self.b_start, self.b_end, self.b_gidx, self.b_aidx) if boundary
                                  else (self.f_start, self.f_end, self.f_gidx, self.f_aidx))
        count = self.nb if boundary else self.n
        start.fill_(-1)
        end.fill_(-1)
        dev = self._device()
        gd = self._griddata(boundary)
        pts = (self.bpos if boundary else self.pos).data_ptr()
        self._launch("assignParticlesToCells", count, struct.pack("<Q", pts), dev, gd)
        keys, perm = self.torch.sort(gidx[:count], stable=True)
        gidx[:count].copy_(keys)
        aidx[:count].copy_(perm.to(self.torch.int32))
        self._launch("calculateCellStartAndEndIndices", count, gd)

    def step(self, dt: float, synchronize: bool = True):
        """SphSimulation::update (SphSimulation.cu:101-120)."""
        n = self.n
        fl, pa = self._fluid(), self._params()
        half = struct.pack("<f", float(np.float32(dt) / np.float32(2.0)))
        self._launch("halfKickVelocities", n, fl, pa, half)
        self._launch("updatePositions", n, fl, self._domain(), struct.pack("<f", float(np.float32(dt))))
        self._update_grid(boundary=False)
        self.density_forces(fl, pa)
        self._launch("halfKickVelocities", n, fl, pa, half)
        if synchronize:
            self.torch.cuda.synchronize()

    def density_forces(self, fl: Optional[bytes] = None, pa: Optional[bytes] = None):
        """The density and acceleration launches of SphSimulation::update (SphSimulation.cu:106-115) on the current
        grid."""
        n = self.n
        fl = fl or self._fluid()
        pa = pa or self._params()
        dev = self._device()
        bd = self._boundary()
        self._launch("computeDensities", n, fl, dev)
        if self.nb:
            self._launch("computeBoundaryDensityContribution", n, fl, bd, dev)
        self._launch("computeExternalAccelerations", n, fl, pa)
        self._launch("computePressureAccelerations", n, fl, dev, pa)
        if self.P.viscosity_constant != 0.0:
            self._launch("computeViscosityAccelerations", n, fl, dev, pa)
        if self.P.surface_tension_constant != 0.0:
            self._launch("computeSurfaceTensionAccelerations", n, fl, dev, pa)
        if self.nb:
            self._launch("computeBoundaryPressureAcceleration", n, fl, bd, dev, pa)
            self._launch("computeBoundaryFrictionAcceleration", n, fl, bd, dev, pa)

    def grid_density_forces(self):
        """The grid build, densities and accelerations of one step on the loaded state (no kicks, no drift)."""
        self._update_grid(boundary=False)
        self.density_forces()
        self.torch.cuda.synchronize()

    def neighbor_total(self) -> int:
        """sumAllNeighbors (Algorithm.cu:234-268) over the current grid: the total the reference's
        calculateAverageNeighborCount divides by the particle count (SphSimulation.cu:237-247)."""
        self.count_buf.zero_()
        self._launch("sumAllNeighbors", self.n, self._fluid(), self._device(),
                     struct.pack("<Q", self.count_buf.data_ptr()))
        self.torch.cuda.synchronize()
        return int(self.count_buf.item()) & 0xFFFFFFFF

    def load(self, arrays: dict):
        """Particle state in slot order (pos, vel, acc (n, 4); rho, rad, h, m (n,))."""
        torch = self.torch
        n = int(arrays["pos"].shape[0])
        if n > self.cap:
            raise ValueError("more particles than capacity")
        self.n = n
        for key, t in (("pos", self.pos), ("vel", self.vel), ("acc", self.acc), ("rho", self.rho), ("rad", self.rad),
                       ("h", self.h), ("m", self.m)):
            t[:n] = torch.from_numpy(np.ascontiguousarray(arrays[key], np.float32)).to(self.dev)
        torch.cuda.synchronize()

    def arrays(self) -> dict:
        self.torch.cuda.synchronize()
        n = self.n
        return {k: t[:n].cpu().numpy().copy() for k, t in (("pos", self.pos), ("vel", self.vel), ("acc", self.acc),
                                                             ("rho", self.rho), ("rad", self.rad), ("h", self.h),
                                                             ("m", self.m))}

    def close(self):
        for m in getattr(self, "modules", {}).values():
            self.drv.cu.cuModuleUnload(m)
        self.modules = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
