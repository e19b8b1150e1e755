"""The C ABI from C++ callers, compiled here with g++: tests/cpp/abi_client.cpp against include/asph.h and
tests/cpp/hpp_client.cpp against the reference-shaped classes of include/asph.hpp. Each generates walls, creates,
steps and exports. The compile and link run on the CPU; the runs need a GPU and are compared bit for bit with the
oracle."""
import os
import subprocess

import numpy as np
import pytest

from adaptivesph_gb300 import _lib
from adaptivesph_gb300.parameters import to_c_parameters
import oracle
from helpers import assert_bitexact, small_dam_break

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", params=["abi_client", "hpp_client"])
def client(request, tmp_path_factory):
    _lib.load()
    lib = _lib.library_path()
    exe = str(tmp_path_factory.mktemp("cpp") / request.param)
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", request.param + ".cpp"), "-o", exe, "-L", libdir,
                    "-lasph_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def test_cpp_client_compiles_and_links(client):
    assert os.path.exists(client)


@pytest.mark.gpu
def test_cpp_client_matches_oracle(client, tmp_path):
    sc = small_dam_break()
    steps = 12
    n = sc.positions.shape[0]
    cp = to_c_parameters(sc.parameters)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(bytes(cp))
        f.write(np.float32(sc.dt).tobytes())
        f.write(np.uint32(steps).tobytes())
        f.write(np.float32(sc.boundary_spacing).tobytes())
        f.write(np.uint32(n).tobytes())
        f.write(np.ascontiguousarray(sc.positions, np.float32).tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([client, str(inp), str(out)], check=True)
    raw = out.read_bytes()
    m = int(np.frombuffer(raw[:4], np.uint32)[0])
    off = 4
    pos = np.frombuffer(raw[off:off + 16 * m], np.float32).reshape(m, 4)
    off += 16 * m
    vel = np.frombuffer(raw[off:off + 16 * m], np.float32).reshape(m, 4)
    off += 16 * m
    rho = np.frombuffer(raw[off:off + 4 * m], np.float32)
    off += 4 * m
    ids = np.frombuffer(raw[off:off + 4 * m], np.uint32)

    bpos, bpsi = oracle.boundary_generate(sc.parameters.domain.min, sc.parameters.domain.max, sc.boundary_spacing,
                                          sc.parameters.rest_density, sc.parameters.base_smoothing_radius)
    orc = oracle.OracleSim(sc.parameters, sc.positions, bpos, bpsi, None, capacity=n)
    for _ in range(steps):
        orc.step(sc.dt)
    o = orc.arrays()
    assert m == orc.n
    assert_bitexact("ids", ids, o["id"])
    assert_bitexact("positions", pos, o["pos"])
    assert_bitexact("velocities", vel, orc.export_velocities())
    assert_bitexact("densities", rho, o["rho"])
