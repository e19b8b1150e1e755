"""adaptivesph_gb300 — GB300-native (sm_103a) implementation of AdaptiveSph's per-step particle pipeline.

The compute path is libasph_gb300.so (hand-written CUDA behind the C ABI of include/asph.h); this package is the
Python mirror of the reference's simulation interface over that ABI, plus headless scene generators.
"""
from .parameters import (BoundaryMode, Criterion, DensityInfo, Domain, Parameters, RefinementParameters,
                         ViscosityModel)
from .simulation import (Batch, BoundaryParticlesDataImportedBuffer, FluidParticlesDataImportedBuffer, ImportedMemory,
                         Server, Simulation, StaticBoundaryDomain, allocate_buffer, create_simulation,
                         create_simulation_with_walls, estimate_device_bytes, import_buffer)
from ._lib import AsphError, load as load_library

__all__ = [
    "AsphError",
    "Batch",
    "BoundaryMode",
    "BoundaryParticlesDataImportedBuffer",
    "Criterion",
    "DensityInfo",
    "Domain",
    "FluidParticlesDataImportedBuffer",
    "ImportedMemory",
    "Parameters",
    "RefinementParameters",
    "Server",
    "Simulation",
    "StaticBoundaryDomain",
    "ViscosityModel",
    "allocate_buffer",
    "create_simulation",
    "create_simulation_with_walls",
    "estimate_device_bytes",
    "import_buffer",
    "load_library",
]
