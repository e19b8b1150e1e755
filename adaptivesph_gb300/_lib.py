"""ctypes binding of libasph_gb300.so (the C ABI declared in include/asph.h).

The library is the only compute path: if it cannot be loaded, or no CUDA device is present, every call that
needs the GPU raises. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import parameters as _p

_lock = threading.Lock()
_lib = None

ASPH_OK = 0
STATUS_NAMES = {
    0: "ok",
    1: "invalid argument",
    2: "CUDA error",
    3: "out of device memory",
    4: "capacity exceeded",
    5: "device check failed",
    6: "unsupported",
    7: "no CUDA device",
}

STAGE_INTEGRATE, STAGE_GRID, STAGE_DENSITY, STAGE_FORCES, STAGE_ALL = 1, 2, 3, 4, 5
KERNEL_CLASSES = ("integrate", "sort", "reorder", "density", "forces", "refine", "refine_merge_select",
                  "refine_merge", "refine_compact", "refine_split_select", "refine_split")

DEVERR_SPIN_LIMIT = 0x1
DEVERR_NONFINITE = 0x2
DEVERR_SPLIT_CAPACITY = 0x4
DEVERR_ID_OVERFLOW = 0x8
DEVERR_ROWS = 0x10


class AsphError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# every function declared in include/asph.h, with its ctypes signature
P = ctypes.POINTER
_vp = ctypes.c_void_p
_u32 = ctypes.c_uint32
_f32 = ctypes.c_float
_fp = P(ctypes.c_float)
_up = P(ctypes.c_uint32)
SIGNATURES = {
    "asph_refinement_parameters_default": (None, [P(_p.CRefinementParameters)]),
    "asph_import_buffer_fd": (ctypes.c_int, [ctypes.c_int, ctypes.c_size_t, P(_vp)]),
    "asph_memory_allocate": (ctypes.c_int, [ctypes.c_size_t, P(_vp)]),
    "asph_memory_device_pointer": (ctypes.c_int, [_vp, P(_vp)]),
    "asph_memory_size": (ctypes.c_int, [_vp, P(ctypes.c_size_t)]),
    "asph_memory_release": (None, [_vp]),
    "asph_boundary_generate": (ctypes.c_int, [P(_p.CDomain), _f32, _f32, _f32, _vp, _u32, _up]),
    "asph_boundary_generate_gpu": (ctypes.c_int, [P(_p.CDomain), _f32, _f32, _f32, _vp, _u32, _up]),
    "asph_simulation_create_with_walls": (ctypes.c_int, [P(_p.CParameters), _fp, _u32, _vp, _vp, _f32,
                                                         P(_p.CRefinementParameters), _u32, _u32, P(_vp)]),
    "asph_simulation_create": (ctypes.c_int, [P(_p.CParameters), _fp, _u32, _vp, _vp, _vp, _u32,
                                              P(_p.CRefinementParameters), _u32, _u32, P(_vp)]),
    "asph_simulation_destroy": (None, [_vp]),
    "asph_simulation_update": (ctypes.c_int, [_vp, _f32]),
    "asph_simulation_step_async": (ctypes.c_int, [_vp, _f32]),
    "asph_simulation_step_cfl": (ctypes.c_int, [_vp, _f32, _f32, _fp]),
    "asph_simulation_synchronize": (ctypes.c_int, [_vp]),
    "asph_simulation_update_domain": (ctypes.c_int, [_vp, P(_p.CDomain), _vp, _u32]),
    "asph_simulation_fluid_count": (ctypes.c_int, [_vp, _up]),
    "asph_simulation_boundary_count": (ctypes.c_int, [_vp, _up]),
    "asph_simulation_average_neighbor_count": (ctypes.c_int, [_vp, _fp]),
    "asph_simulation_density_info": (ctypes.c_int, [_vp, _f32, P(_p.CDensityInfo)]),
    "asph_simulation_enable_adaptive_refinement": (ctypes.c_int, [_vp]),
    "asph_simulation_export": (ctypes.c_int, [_vp]),
    "asph_simulation_export_host": (ctypes.c_int, [_vp, _fp, _fp, _fp, _fp, _up, _u32]),
    "asph_simulation_export_host_async": (ctypes.c_int, [_vp, _fp, _fp, _fp, _fp, _up, _u32]),
    "asph_simulation_export_wait": (ctypes.c_int, [_vp]),
    "asph_simulation_totals": (ctypes.c_int, [_vp, P(_p.CTotals)]),
    "asph_simulation_device_errors": (ctypes.c_int, [_vp, _up, ctypes.c_int]),
    "asph_simulation_set_stream": (ctypes.c_int, [_vp, _vp]),
    "asph_simulation_state_info": (ctypes.c_int, [_vp, P(_p.CStateInfo)]),
    "asph_simulation_read_fluid": (ctypes.c_int, [_vp, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _up, _u32]),
    "asph_simulation_write_fluid": (ctypes.c_int, [_vp, P(_p.CStateInfo), _fp, _fp, _fp, _fp, _fp, _fp, _fp, _up]),
    "asph_simulation_run_stages": (ctypes.c_int, [_vp, _f32, _u32]),
    "asph_simulation_grid_info": (ctypes.c_int, [_vp, P(_p.CGridInfo)]),
    "asph_simulation_read_grid": (ctypes.c_int, [_vp, _up, _u32, _up, _up, _u32]),
    "asph_simulation_neighbor_counts": (ctypes.c_int, [_vp, _up, _u32]),
    "asph_simulation_last_refinement": (ctypes.c_int, [_vp, P(_p.CRefinementReport)]),
    "asph_simulation_enable_timing": (ctypes.c_int, [_vp, ctypes.c_int]),
    "asph_simulation_kernel_times": (ctypes.c_int, [_vp, P(ctypes.c_double), _up, _u32]),
    "asph_simulation_launch_count": (ctypes.c_int, [_vp, P(ctypes.c_uint64)]),
    "asph_simulation_device_bytes": (ctypes.c_int, [_vp, P(ctypes.c_uint64)]),
    "asph_estimate_device_bytes": (ctypes.c_int, [P(_p.CParameters), _u32, _u32, P(_p.CRefinementParameters), _u32,
                                                  _u32, P(ctypes.c_uint64)]),
    "asph_server_create": (ctypes.c_int, [ctypes.c_uint64, _u32, P(_vp)]),
    "asph_server_destroy": (None, [_vp]),
    "asph_server_submit": (ctypes.c_int, [_vp, P(_p.CRequest), P(ctypes.c_uint64)]),
    "asph_server_poll": (ctypes.c_int, [_vp, _u32, P(_u32)]),
    "asph_server_status": (ctypes.c_int, [_vp, ctypes.c_uint64, P(_p.CRequestStatus)]),
    "asph_server_take": (ctypes.c_int, [_vp, ctypes.c_uint64, _fp, _fp, _fp, _fp, _up, _u32]),
    "asph_server_stats": (ctypes.c_int, [_vp, P(ctypes.c_uint64), P(_u32), P(_u32), P(ctypes.c_uint64),
                                         P(ctypes.c_uint64)]),
    "asph_batch_create": (ctypes.c_int, [P(_vp), _u32, P(_vp)]),
    "asph_batch_destroy": (None, [_vp]),
    "asph_batch_step": (ctypes.c_int, [_vp, _fp, _u32]),
    "asph_batch_stats": (ctypes.c_int, [_vp, P(ctypes.c_uint64), P(ctypes.c_uint64), P(ctypes.c_uint64)]),
    "asph_batch_set_mode": (ctypes.c_int, [_vp, _u32]),
    "asph_batch_tuning": (ctypes.c_int, [_vp, _vp]),
    "asph_grid_sort_noalloc": (ctypes.c_int, [P(_p.CParameters), _vp, _u32, _vp, _vp, _vp, _vp, _u32, _vp, _vp]),
    "asph_abi_version": (ctypes.c_uint32, []),
    "asph_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "asph_last_error": (ctypes.c_char_p, []),
}

# test hooks exported by the library but not part of the public header
DEBUG_SIGNATURES = {
    "asph_debug_record_refinement": (ctypes.c_int, [_vp, ctypes.c_int]),
    "asph_debug_refinement_ids": (ctypes.c_int, [_vp, _up, _up, _up, _u32]),
    "asph_debug_wait_limit_probe": (ctypes.c_int, [_up]),
    "asph_debug_host_reads_in_place": (ctypes.c_int, [ctypes.c_int]),
}


def library_path() -> str:
    from . import build as _build

    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads (building first if needed) the CUDA library. Raises if it cannot be built or loaded."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        from . import build as _build

        path = _build.LIB
        if build_if_missing and _build.needs_build():
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"libasph_gb300.so not found at {path}; run adaptivesph_gb300.build.build()")
        lib = ctypes.CDLL(path)
        for name, (res, args) in {**SIGNATURES, **DEBUG_SIGNATURES}.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int, where: str) -> None:
    if status != ASPH_OK:
        msg = _lib.asph_last_error().decode(errors="replace") if _lib is not None else ""
        raise AsphError(status, where, msg)
