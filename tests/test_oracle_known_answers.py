"""The oracle against answers known independently of it (CPU only).

The reference ships no golden vectors for this path, so the oracle is pinned by analytic facts and by
independent numpy restatements: the Wendland kernel's normalisation and derivative, the density of a perfect
lattice, the split directions, the correctly rounded cube root, the stable sort, Morton keys, the reference's
excluded-cell quirk, and the refinement bookkeeping."""
import ctypes
import math

import numpy as np
import pytest

import oracle
from adaptivesph_gb300 import scenes
from adaptivesph_gb300.parameters import Criterion, RefinementParameters

L = oracle.lib()


def wendland_np(r, h):
    """W(r, h) = 21/(16 pi h^3) (1 - q/2)^4 (2q + 1), q = r/h <= 2 (WendlandKernel.cuh:39-52), FP64."""
    q = np.asarray(r, np.float64) / h
    w = 21.0 / (16.0 * math.pi * h ** 3) * (1.0 - q / 2.0) ** 4 * (2.0 * q + 1.0)
    return np.where(q <= 2.0, w, 0.0)


@pytest.mark.parametrize("h", [0.0052, 0.013, 1.0])
def test_kernel_integrates_to_one(h):
    r = np.linspace(0.0, 2.0 * h, 200001)
    w = np.array([L.orc64_kernel_w(x, h) for x in r[::100]])
    np.testing.assert_allclose(w, wendland_np(r[::100], h), rtol=1e-12, atol=1e-14 * wendland_np(0.0, h))
    wf = np.array([L.orc64_kernel_w(x, h) for x in r])
    integral = np.trapezoid(4.0 * math.pi * r * r * wf, r)
    assert integral == pytest.approx(1.0, abs=1e-8)
    assert L.orc64_kernel_w(2.0 * h * 1.0001, h) == 0.0


def test_kernel_derivative_matches_finite_difference():
    h = 0.013
    for r in np.linspace(0.05 * h, 1.95 * h, 37):
        e = 1e-7 * h
        fd = (L.orc64_kernel_w(r + e, h) - L.orc64_kernel_w(r - e, h)) / (2 * e)
        assert L.orc64_kernel_dw(r, h) == pytest.approx(fd, rel=1e-6, abs=1e-9 / h ** 4)


def test_kernel_fp32_close_to_fp64():
    h = np.float32(0.0052)
    for r in np.linspace(0.0, 2.0 * float(h), 101, dtype=np.float32):
        w32 = L.orc32_kernel_w(float(r), float(h))
        w64 = L.orc64_kernel_w(float(r), float(h))
        assert abs(w32 - w64) <= 2e-6 * L.orc64_kernel_w(0.0, float(h))


def test_lattice_density_matches_direct_sum():
    """Interior particles of a perfect lattice: the oracle's neighbour search + kernel sum equals a brute-force
    numpy sum over every lattice point, and is close to the rest density."""
    sc = scenes.dam_break((14, 14, 14), 0.01, seed=1, jitter=0.0, tank=(0.6, 0.6, 0.6), walls=False)
    p = sc.parameters
    o = oracle.OracleSim(p, sc.positions)
    o.grid_build()
    rho32 = o.density32()
    rho64 = o.density64()
    pos = o.arrays()["pos"][:, :3].astype(np.float64)
    centre = pos.mean(axis=0)
    inner = np.where(np.abs(pos - centre).max(axis=1) < 0.02)[0]
    assert inner.size > 0
    h = float(np.float32(p.base_smoothing_radius))
    m = float(np.float32(p.base_particle_mass))
    for i in inner:
        d = np.linalg.norm(pos - pos[i], axis=1)
        want = m * wendland_np(d, h).sum()
        assert rho64[i] == pytest.approx(want, rel=1e-12)
        assert rho32[i] == pytest.approx(want, rel=1e-5)
        assert want == pytest.approx(p.rest_density, rel=0.02)


def test_split_directions_are_the_icosahedron():
    v = np.zeros(36, np.float32)
    L.orc_icosahedron(v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    v = v.reshape(12, 3).astype(np.float64)
    np.testing.assert_allclose(np.linalg.norm(v, axis=1), 1.0, atol=1e-6)
    np.testing.assert_allclose(v.sum(axis=0), 0.0, atol=1e-6)
    d = v @ v.T
    np.fill_diagonal(d, -2)
    # every vertex has 5 nearest neighbours at cos = 1/sqrt(5) and one antipode
    for row in d:
        assert np.sum(np.isclose(row, 1 / math.sqrt(5), atol=1e-6)) == 5
        assert np.sum(np.isclose(row, -1.0, atol=1e-6)) == 1
    phi = (1 + math.sqrt(5)) / 2
    inv = 1 / math.sqrt(1 + phi * phi)
    np.testing.assert_allclose(v[0], [0.0, phi * inv, inv], atol=1e-6)


def test_cbrt_is_correctly_rounded():
    rng = np.random.default_rng(5)
    x = (rng.uniform(0.5, 1.0, 20000) * np.exp2(rng.integers(-40, 40, 20000))).astype(np.float32)
    x = np.concatenate([x, np.float32([1.0, 8.0, 0.001, 0.077, 1e-30, 3.0e30])])
    got = np.array([oracle.cbrtf(float(v)) for v in x], np.float32)
    # cbrt in FP64 then rounded to float is correctly rounded unless the FP64 value sits within 2^-52 of a
    # rounding boundary; none of these inputs does
    want = np.cbrt(x.astype(np.float64)).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_sort_is_stable():
    rng = np.random.default_rng(9)
    for n, bits in [(1, 8), (1000, 8), (50000, 24), (70000, 30)]:
        key = rng.integers(0, min(1 << bits, 300), n).astype(np.uint32)
        perm = np.zeros(n, np.uint32)
        L.orc_sort_stable(n, oracle.uptr(key), bits, oracle.uptr(perm))
        assert np.array_equal(perm, np.argsort(key, kind="stable").astype(np.uint32))


def _morton_py(x, y, z):
    k = 0
    for b in range(10):
        k |= ((x >> b) & 1) << (3 * b) | ((y >> b) & 1) << (3 * b + 1) | ((z >> b) & 1) << (3 * b + 2)
    return k


def test_morton_keys():
    rng = np.random.default_rng(3)
    for x, y, z in rng.integers(0, 1024, (500, 3)):
        assert L.orc_morton3(int(x), int(y), int(z)) == _morton_py(int(x), int(y), int(z))


def _excluded(refkeys, slots):
    rk = np.asarray(refkeys, np.uint32)
    sl = np.asarray(slots, np.uint32)
    ex = (ctypes.c_uint32 * 2)()
    L.orc_excluded_cells(len(rk), oracle.uptr(rk), oracle.uptr(sl), ex)
    return tuple(int(v) for v in ex)


def test_excluded_cells_quirk():
    NONE = 0xFFFFFFFF
    # one particle: its cell has no valid range (NeighborKernels.cu:17-44)
    assert _excluded([7], [0]) == (7, NONE)
    # the first two of the (cell, slot) order in different cells: both cells are skipped
    assert _excluded([9, 3, 5, 3], [0, 1, 2, 3]) == (NONE, NONE)
    assert _excluded([9, 3, 5], [0, 1, 2]) == (3, 5)
    # the first two share a cell: nothing is skipped
    assert _excluded([4, 4, 8], [2, 0, 1]) == (NONE, NONE)
    assert _excluded([], []) == (NONE, NONE)


def test_refinement_bookkeeping():
    """A refinement pass: counts add up (n' = n - removed + 12 splits) and the mass changes by exactly the
    reference's split ratio (13 x 0.077 = 1.001 of each parent, Q-7) with merges conserving mass."""
    ref = RefinementParameters(enabled=True, min_mass_ratio=0.05, max_mass_ratio=8.0, max_particle_count=40000,
                               max_batch_ratio=0.2, initial_cooldown=2, cooldown=3, criterion=Criterion.VELOCITY)
    ref.velocity_split_min_speed = 0.05
    ref.velocity_merge_max_speed = 0.2
    sc = scenes.dam_break((10, 20, 10), 0.02, seed=11, tank=(0.6, 0.6, 0.4), refinement=ref)
    bd_pos, bd_psi = oracle.boundary_generate(sc.parameters.domain.min, sc.parameters.domain.max,
                                              sc.boundary_spacing, sc.parameters.rest_density,
                                              sc.parameters.base_smoothing_radius)
    o = oracle.OracleSim(sc.parameters, sc.positions, bd_pos, bd_psi, ref)
    seen_split = False
    for _ in range(12):
        before = o.arrays()
        m_by_id = dict(zip(before["id"].tolist(), before["m"].astype(np.float64).tolist()))
        if not o.step(sc.dt):
            continue
        r = o.last_report()
        assert r["count_after"] == r["count_before"] - r["removed"] + 12 * r["splits"]
        assert r["removed"] == r["merge_pairs"]
        assert r["splits"] <= max(r["split_budget"], 0) + 255  # Q-8: up to a block of extra splits
        mass_before = sum(m_by_id.values())
        mass_after = float(o.arrays()["m"].astype(np.float64).sum())
        gain = sum(0.001 * m_by_id[int(p)] for p in r["split_ids"])
        assert mass_after == pytest.approx(mass_before + gain, rel=1e-6)
        seen_split |= r["splits"] > 0
    assert seen_split
