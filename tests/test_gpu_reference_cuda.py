"""The reference's own CUDA kernels run on the GPU (oracle/ref_cuda.py: cubins built from the reference's sources,
launched through the driver API) against the reference's results run on the CPU (golden fixtures written by
tests/golden/make_ref_golden.py) and against the oracle: this validates the reference arm's GPU leg before its
timings are used.

Tolerances: the GPU build of the reference contracts multiply-adds (nvcc's default, as the reference's own build
does) and uses CUDA's powf and sqrtf, where the CPU build rounds every operation (-ffp-contract=off) and uses the
host's, so results agree to FP32 rounding, not bit for bit: densities within 1e-5 relative, accelerations within
2e-5 of the FP64 sum of |pair terms| + |g|; the neighbour total may differ by pairs whose distance lies within
rounding of the support radius (at most 4 of ~10^5 here)."""
import os

import numpy as np
import pytest

import oracle
from adaptivesph_gb300 import scenes
from helpers import boundary_of, small_dam_break
from oracle import ref_cuda

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available(), reason="the reference's cubins are not built here")]

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _state_by_id(sc, steps):
    bd = boundary_of(sc)
    nb = bd.get_particle_count()
    o = oracle.OracleSim(sc.parameters, sc.positions, bd.positions if nb else None, bd.psi if nb else None, None,
                         capacity=sc.positions.shape[0])
    for _ in range(steps):
        o.step(sc.dt)
    st = o.arrays()
    order = np.argsort(st["id"], kind="stable")
    return {k: v[order] for k, v in st.items()}, bd


def _against_fixture(sc, fixture):
    g = np.load(os.path.join(GOLDEN, fixture))
    st, bd = _state_by_id(sc, int(g["steps"]))
    nb = bd.get_particle_count()
    r = ref_cuda.RefCudaSim(sc.parameters, st["pos"], bd.positions if nb else None, bd.psi if nb else None)
    r.load(st)
    r.grid_density_forces()
    got = r.arrays()
    idx = np.searchsorted(st["id"], g["id"])  # slots are in id order
    assert np.array_equal(st["id"][idx], g["id"])
    np.testing.assert_allclose(got["rho"][idx], g["rho"], rtol=1e-5)
    err = np.abs(got["acc"][idx, :3].astype(np.float64) - g["acc"]).max(axis=1)
    worst = float((err / g["scale"]).max())
    assert worst <= 2e-5, worst
    total = r.neighbor_total()
    r.close()
    return total, g


def test_reference_gpu_kernels_match_reference_cpu_small_tank():
    total, g = _against_fixture(small_dam_break(), "reference_kernels_small_tank.npz")
    want = int(g["counts"].astype(np.int64).sum())
    assert abs(total - want) <= 4, (total, want)


def test_reference_gpu_kernels_match_reference_cpu_128k_sample():
    _against_fixture(scenes.c1_plain(), "reference_kernels_c1_sample.npz")


def test_reference_gpu_trajectory_tracks_oracle():
    """20 plain steps from the same lattice, each side on its own: the reference's GPU trajectory and the oracle's
    stay within FP32 rounding of each other."""
    sc = small_dam_break()
    bd = boundary_of(sc)
    nb = bd.get_particle_count()
    o = oracle.OracleSim(sc.parameters, sc.positions, bd.positions if nb else None, bd.psi if nb else None, None,
                         capacity=sc.positions.shape[0])
    r = ref_cuda.RefCudaSim(sc.parameters, sc.positions, bd.positions if nb else None, bd.psi if nb else None)
    for _ in range(20):
        o.step(sc.dt)
        r.step(sc.dt)
    a = o.arrays()
    order = np.argsort(a["id"], kind="stable")
    v = o.export_velocities()[order]
    b = r.arrays()
    np.testing.assert_allclose(b["pos"][:, :3], a["pos"][order, :3], atol=1e-5)
    np.testing.assert_allclose(b["rho"], a["rho"][order], rtol=1e-4)
    vmax = np.abs(v).max()
    np.testing.assert_allclose(b["vel"][:, :3], v[:, :3], atol=1e-3 * vmax)
    r.close()
