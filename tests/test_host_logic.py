"""Host-side logic on the CPU: scene generators, parameter conversion, and the bench's aggregation of independent
replicas across ranks (world size 2 over gloo)."""
import os
import socket

import numpy as np
import pytest

import bench
from adaptivesph_gb300 import scenes
from adaptivesph_gb300.parameters import to_c_parameters


def test_scenes_are_seeded_and_sized():
    a = scenes.c1_plain()
    b = scenes.c1_plain()
    assert a.positions.shape == (128000, 4)
    assert np.array_equal(a.positions, b.positions)
    c = scenes.c1_plain(seed=2)
    assert not np.array_equal(a.positions, c.positions)
    # jitter stays within +-0.05 dx of the lattice
    dx = 0.01
    frac = a.positions[:, :3] / dx - 0.5
    assert np.abs(frac - np.round(frac)).max() <= 0.05 + 1e-4
    p = a.parameters
    assert p.base_smoothing_radius == pytest.approx(1.3 * dx)
    assert p.speed_of_sound == pytest.approx(10 * np.sqrt(2 * 9.81 * 0.8))


def test_c2_workload_definition():
    sc = scenes.c2_adaptive()
    assert sc.positions.shape[0] == 1_000_000
    r = sc.refinement
    assert r.enabled and r.max_particle_count == 4_000_000
    assert r.min_mass_ratio == pytest.approx(0.05) and r.max_mass_ratio == pytest.approx(8.0)
    assert r.initial_cooldown == 10 and r.cooldown == 10


def test_parameter_conversion_keeps_values():
    sc = scenes.taylor_green(16)
    c = to_c_parameters(sc.parameters)
    assert c.boundary_mode == 1 and c.viscosity_model == 1
    assert c.kinematic_viscosity == pytest.approx(sc.parameters.kinematic_viscosity)
    assert tuple(c.domain.max) == pytest.approx(tuple(sc.parameters.domain.max))


def test_replica_throughput_single_rank():
    rows = np.array([[1000.0, 0.5, 400.0, 2.0]])
    v, e = bench.replica_throughput(rows)
    assert v == pytest.approx(2000.0) and e == pytest.approx(200.0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _replica_worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [1000.0 * (rank + 1), 0.5 + rank, 100.0 * (rank + 1), 1.0 + rank]
        rows = bench.gather_rows(local, dist, world, "cpu")
        out[rank] = bench.replica_throughput(rows)
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_gloo_world_size_2():
    """Two ranks over gloo: whole-job value = all ranks' particle-steps over the slowest rank's time."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        v, e = res[r]
        assert v == pytest.approx((1000.0 + 2000.0) / 1.5)
        assert e == pytest.approx((100.0 + 200.0) / 2.0)
