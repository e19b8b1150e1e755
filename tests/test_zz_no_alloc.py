"""asph_grid_sort_noalloc (the cell sort with a fixed scratch array, no allocation) against the simulation's own
grid build, through the C ABI. Collected last so that it also runs after every other GPU test in one process."""
import ctypes

import numpy as np
import pytest

from adaptivesph_gb300 import _lib
from adaptivesph_gb300.parameters import to_c_parameters
from helpers import assert_bitexact, make_pair, small_dam_break

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc_sort(params, pos4: np.ndarray, cell_count: int):
    """Runs the entry point on device copies of pos4; returns (sorted keys, order, start, end, device errors)."""
    L = _lib.load()
    n = pos4.shape[0]
    dev = torch.device("cuda:0")
    d_pos = torch.from_numpy(np.ascontiguousarray(pos4, np.float32)).to(dev)
    d_keys = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    d_order = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    d_start = torch.empty(cell_count, dtype=torch.int32, device=dev)
    d_end = torch.empty(cell_count, dtype=torch.int32, device=dev)
    d_err = torch.zeros(1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    cp = to_c_parameters(params)
    st = L.asph_grid_sort_noalloc(ctypes.byref(cp), d_pos.data_ptr(), n, d_keys.data_ptr(), d_order.data_ptr(),
                                  d_start.data_ptr(), d_end.data_ptr(), cell_count, d_err.data_ptr(), None)
    _lib.check(st, "asph_grid_sort_noalloc")
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)
    return u(d_keys)[:n], u(d_order)[:n], u(d_start), u(d_end), int(u(d_err)[0])


def _check_against_simulation(sim, params, pos4):
    info = sim.grid_info()
    keys, start, end = sim.read_grid()
    sorted_pos = sim.read_state()["pos"]
    got_keys, order, got_start, got_end, err = _noalloc_sort(params, pos4, int(info["cell_count"]))
    assert err == 0
    assert_bitexact("sorted keys", got_keys, keys)
    assert_bitexact("sorted positions", pos4[order], sorted_pos)
    assert_bitexact("cell_start", got_start, start)
    assert_bitexact("cell_end", got_end, end)
    # stable: the order is the stable argsort of the input's keys
    input_keys = np.empty_like(got_keys)
    input_keys[order] = got_keys
    assert_bitexact("order", order, np.argsort(input_keys, kind="stable").astype(np.uint32))


def test_noalloc_sort_matches_simulation_grid_two_calls():
    sc = small_dam_break()
    sim, _ = make_pair(sc)
    pos4 = np.ascontiguousarray(sc.positions.reshape(-1, 4), np.float32)
    # call 1: the caller's initial positions against a grid build of the unchanged state (dt = 0 moves nothing)
    sim.run_stages(0.0, _lib.STAGE_GRID)
    _check_against_simulation(sim, sc.parameters, pos4)
    # call 2, right after: positions after a few steps (cell-sorted by the step's grid build)
    for _ in range(5):
        sim.update(sc.dt)
    _check_against_simulation(sim, sc.parameters, np.ascontiguousarray(sim.read_state()["pos"]))


def test_noalloc_sort_at_the_limit_three_digit_passes_no_device_memory_change():
    """ASPH_NOALLOC_MAX_PARTICLES seeded random positions in the reference's 1.6 x 1.0 x 0.67 m tank at dx = 0.01 m
    (62 x 40 x 26 sub-cells: 18-bit keys, three digit passes, so the sorted result comes back out of the scratch half
    and 171 tiles exercise the look-back across tiles), against the simulation's grid build of the same positions;
    two calls in a row, with the device's free memory unchanged across both."""
    from adaptivesph_gb300 import StaticBoundaryDomain, create_simulation, scenes

    limit = 524288
    sc = scenes.dam_break((40, 80, 40), 0.01, seed=1)
    d = sc.parameters.domain
    rng = np.random.default_rng(7)
    lo = np.array(d.min, np.float32)
    hi = np.array(d.max, np.float32)
    pos4 = np.zeros((limit, 4), np.float32)
    pos4[:, :3] = (lo + (hi - lo) * rng.random((limit, 3), dtype=np.float32)).astype(np.float32)
    sim = create_simulation(sc.parameters, pos4, None, None, StaticBoundaryDomain.empty(d), None, limit, 1)
    info = sim.grid_info()
    assert int(info["key_bits"]) > 16, "three digit passes wanted"
    sim.run_stages(0.0, _lib.STAGE_GRID)
    _check_against_simulation(sim, sc.parameters, pos4)  # also loads the library's device code, if not yet
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        got_keys, order, got_start, got_end, err = _noalloc_sort(sc.parameters, pos4, int(info["cell_count"]))
        assert err == 0
        keys, start, end = sim.read_grid()
        assert_bitexact("sorted keys", got_keys, keys)
        assert_bitexact("cell_start", got_start, start)
        assert_bitexact("cell_end", got_end, end)
        input_keys = np.empty_like(got_keys)
        input_keys[order] = got_keys
        assert_bitexact("order", order, np.argsort(input_keys, kind="stable").astype(np.uint32))
    torch.cuda.synchronize()
    # the device arrays of _noalloc_sort are freed back to torch's cache, not to the device: the driver's free
    # memory moves only if something allocated device memory
    assert torch.cuda.mem_get_info()[0] == free0
    sim.close()


def test_noalloc_sort_rejects_count_above_limit():
    sc = small_dam_break()
    L = _lib.load()
    cp = to_c_parameters(sc.parameters)
    limit = 524288
    st = L.asph_grid_sort_noalloc(ctypes.byref(cp), None, limit + 1, None, None, None, None, 0, None, None)
    assert st != 0
    st = L.asph_grid_sort_noalloc(ctypes.byref(cp), 16, limit + 1, 16, 16, None, None, 0, 16, None)
    assert st == 4  # ASPH_ERR_CAPACITY
    assert b"fixed scratch limit" in L.asph_last_error()
