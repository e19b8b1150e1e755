"""The committed golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py from the oracle):
the oracle re-run here must reproduce them bit for bit (a change of its arithmetic or order shows up first here),
and the CUDA pipeline must reproduce them bit for bit on the GPU, through the C ABI."""
import importlib.util
import os

import numpy as np
import pytest

from adaptivesph_gb300 import create_simulation
from helpers import assert_bitexact, boundary_of

HERE = os.path.dirname(os.path.abspath(__file__))
_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
make_golden = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(make_golden)
CASES = make_golden.cases()


def golden(name):
    with np.load(os.path.join(HERE, "golden", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def compare(got, want):
    assert got["pos"].shape == want["pos"].shape
    for k in ("pos", "rho", "h", "m", "id", "export_vel"):
        assert_bitexact(k, got[k], want[k])


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(name):
    scene, steps = CASES[name]
    want = golden(name)
    assert int(want["steps"]) == steps
    compare(make_golden.run_oracle(scene, steps), want)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_reproduces_golden(name):
    scene, steps = CASES[name]
    want = golden(name)
    bd = boundary_of(scene)
    n = scene.positions.shape[0]
    cap = scene.refinement.max_particle_count if scene.refinement else n
    sim = create_simulation(scene.parameters, scene.positions, None, None, bd, scene.refinement, cap,
                            max(bd.get_particle_count(), 1))
    if scene.velocities is not None:
        st = sim.read_state()
        st["vel"] = scene.velocities.copy()
        sim.write_state(st, next_id=n)
    for _ in range(steps):
        sim.step_async(scene.dt)
    sim.synchronize()
    st = sim.read_state()
    got = {k: st[k] for k in ("pos", "rho", "h", "m", "id")}
    got["export_vel"] = sim.export_host()["velocities"]
    compare(got, want)
    sim.close()
