"""The C ABI on the CPU: the library loads and exports every function include/asph.h declares, the ctypes
declarations match the header (names and struct layouts, checked against gcc's own layout), and the host-only
entry points (status strings, refinement defaults, boundary generation) behave. No call here touches a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from adaptivesph_gb300 import _lib
from adaptivesph_gb300 import parameters as P
from adaptivesph_gb300.parameters import Domain

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "asph.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_]\w*\s*\*?\s*(asph_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_header_declares_the_reference_interface():
    names = header_functions()
    for must in ("asph_simulation_create", "asph_simulation_update", "asph_simulation_update_domain",
                 "asph_simulation_fluid_count", "asph_simulation_boundary_count",
                 "asph_simulation_average_neighbor_count", "asph_simulation_density_info",
                 "asph_simulation_enable_adaptive_refinement", "asph_import_buffer_fd", "asph_boundary_generate",
                 "asph_grid_sort_noalloc"):
        assert must in names


def test_library_exports_every_header_function(lib):
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_the_header():
    assert sorted(_lib.SIGNATURES) == header_functions()


STRUCTS = {
    "asph_domain": P.CDomain,
    "asph_parameters": P.CParameters,
    "asph_refinement_parameters": P.CRefinementParameters,
    "asph_boundary_particle": P.CBoundaryParticle,
    "asph_density_info": P.CDensityInfo,
    "asph_totals": P.CTotals,
    "asph_state_info": P.CStateInfo,
    "asph_grid_info": P.CGridInfo,
    "asph_refinement_report": P.CRefinementReport,
    "asph_request": P.CRequest,
    "asph_request_status": P.CRequestStatus,
}


def test_struct_layouts_match_the_compiler(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void) {"]
    for cname, cls in STRUCTS.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for cname, cls in STRUCTS.items():
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(cls, fname).offset, (cname, fname)


def test_status_strings(lib):
    for s in range(8):
        assert lib.asph_status_string(s)
    assert lib.asph_abi_version() == 1


def test_refinement_defaults_are_the_reference_defaults(lib):
    """RefinementParameters.cuh:8-104 defaults."""
    r = P.CRefinementParameters()
    lib.asph_refinement_parameters_default(ctypes.byref(r))
    f = np.float32
    assert r.enabled == 0
    assert f(r.min_mass_ratio) == f(0.3) and f(r.max_mass_ratio) == f(8.0)
    assert r.max_particle_count == 1000000 and f(r.max_batch_ratio) == f(0.2)
    assert r.initial_cooldown == 10 and r.cooldown == 10 and r.criterion == 0
    assert f(r.split_epsilon) == f(0.65) and f(r.split_alpha) == f(0.70)
    assert f(r.split_center_mass_ratio) == f(0.077) and f(r.split_vertex_mass_ratio) == f(0.077)
    assert f(r.velocity_split_min_speed) == f(2.0) and f(r.velocity_merge_max_speed) == f(0.1)
    assert f(r.vorticity_split_min) == f(1.0) and f(r.vorticity_merge_max) == f(0.3)
    assert f(r.curvature_split_min) == f(2.0) and f(r.curvature_merge_max) == f(0.6)
    assert f(r.interface_split_distance_ratio) == f(0.05) and f(r.interface_merge_distance_ratio) == f(0.15)


@pytest.mark.parametrize("tank,spacing,h", [((0.6, 0.6, 0.4), 0.02, 0.026), ((1.6, 1.0, 0.67), 0.01, 0.013)])
def test_boundary_generation_matches_oracle(tank, spacing, h):
    """StaticBoundaryDomain::generate (host code of the product) against its restatement, bit for bit."""
    from adaptivesph_gb300 import StaticBoundaryDomain

    d = Domain(min=(0.0, 0.0, 0.0), max=tank, friction=0.01)
    bd = StaticBoundaryDomain.generate(d, spacing, 1000.0, h)
    pos, psi = oracle.boundary_generate(d.min, d.max, spacing, 1000.0, h)
    assert bd.get_particle_count() == pos.shape[0]
    assert np.array_equal(bd.positions.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(bd.psi.view(np.uint32), psi.view(np.uint32))


def test_boundary_generation_reports_capacity(lib):
    d = P.to_c_domain(Domain(min=(0.0, 0.0, 0.0), max=(0.3, 0.3, 0.3), friction=0.01))
    n = ctypes.c_uint32()
    assert lib.asph_boundary_generate(ctypes.byref(d), 0.02, 1000.0, 0.026, None, 0, ctypes.byref(n)) == 0
    assert n.value > 0
    small = (P.CBoundaryParticle * 4)()
    st = lib.asph_boundary_generate(ctypes.byref(d), 0.02, 1000.0, 0.026, small, 4, ctypes.byref(n))
    assert st == 4  # ASPH_ERR_CAPACITY
