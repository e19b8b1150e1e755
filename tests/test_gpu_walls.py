"""StaticBoundaryDomain::generate on the GPU (asph_boundary_generate_gpu, asph_simulation_create_with_walls, walls of
served requests) against the host generator, bit for bit: wall positions and psi, and the simulations and served
results built on them."""
import numpy as np
import pytest

from adaptivesph_gb300 import Server, StaticBoundaryDomain, create_simulation, create_simulation_with_walls, scenes
from helpers import assert_bitexact, boundary_of, small_dam_break

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tank,dx,spacing_ratio", [
    ((0.6, 0.6, 0.4), 0.02, 1.0),       # small tank, walls within 2h of the fluid
    ((1.6, 1.0, 0.67), 0.01, 1.0),      # the 128k dam break's tank (80k walls)
    ((1.6, 1.0, 0.67), 0.004, 1.0),     # the 1M adaptive dam break's tank (503k walls)
    ((0.5, 0.5, 0.35), 0.02, 1.0 / 8),  # dense walls: hundreds of wall neighbours per wall particle
])
def test_gpu_walls_equal_host_walls(tank, dx, spacing_ratio):
    sc = scenes.dam_break((4, 4, 4), dx, tank=tank)
    p = sc.parameters
    args = (p.domain, sc.boundary_spacing * spacing_ratio, p.rest_density, p.base_smoothing_radius)
    host = StaticBoundaryDomain.generate(*args)
    gpu = StaticBoundaryDomain.generate(*args, device=True)
    assert host.get_particle_count() > 1000
    assert_bitexact("wall positions", gpu.positions, host.positions)
    assert_bitexact("psi", gpu.psi, host.psi)


def test_simulation_with_device_walls_equals_host_walls():
    sc = small_dam_break()
    a = create_simulation(sc.parameters, sc.positions, None, None, boundary_of(sc), None, sc.positions.shape[0], 1)
    b = create_simulation_with_walls(sc.parameters, sc.positions, sc.boundary_spacing, None, sc.positions.shape[0])
    assert a.get_boundary_particles_count() == b.get_boundary_particles_count() > 0
    for _ in range(10):
        a.update(sc.dt)
        b.update(sc.dt)
    sa, sb = a.read_state(), b.read_state()
    for k in ("pos", "vel", "acc", "rho", "id"):
        assert_bitexact(k, sb[k], sa[k])


def test_served_request_with_device_walls_equals_explicit_walls():
    sc = small_dam_break()
    server = Server(8 << 30)
    t1 = server.submit(sc.parameters, sc.positions, boundary_of(sc), None, sc.dt, 15)
    t2 = server.submit(sc.parameters, sc.positions, None, None, sc.dt, 15, wall_spacing=sc.boundary_spacing)
    while server.poll(5):
        pass
    a, b = server.take(t1), server.take(t2)
    for k in ("ids", "positions", "velocities", "densities", "radii"):
        assert_bitexact(k, b[k], a[k])
    server.close()
