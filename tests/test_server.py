"""The serving loop: requests admitted under a device-memory budget, run together, retired; each result equals the
request run alone, bit for bit, and the budget is never exceeded."""
import numpy as np
import pytest

from adaptivesph_gb300 import Server, create_simulation, estimate_device_bytes
from helpers import adaptive_refinement, assert_bitexact, boundary_of, small_dam_break



def _requests():
    return [
        (small_dam_break(), 30),
        (small_dam_break(counts=(8, 12, 8), seed=3), 45),
        (small_dam_break(refinement=adaptive_refinement()), 25),
        (small_dam_break(counts=(12, 16, 8), seed=5, refinement=adaptive_refinement(cooldown=4)), 40),
        (small_dam_break(counts=(6, 10, 6), seed=8), 12),
    ]


def _alone(sc, steps):
    bd = boundary_of(sc)
    cap = sc.refinement.max_particle_count if sc.refinement else sc.positions.shape[0]
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd, sc.refinement, cap,
                            max(bd.get_particle_count(), 1))
    for _ in range(steps):
        sim.update(sc.dt)
    out = sim.export_host()
    sim.close()
    return out


def _bytes(sc):
    bd = boundary_of(sc)
    cap = sc.refinement.max_particle_count if sc.refinement else sc.positions.shape[0]
    return estimate_device_bytes(sc.parameters, sc.positions.shape[0], bd.get_particle_count(), sc.refinement, cap)


@pytest.mark.gpu
def test_server_results_equal_alone_under_a_budget():
    reqs = _requests()
    sizes = [_bytes(sc) for sc, _ in reqs]
    budget = int(sum(sorted(sizes)[-2:]) * 1.01)  # room for about two requests at a time: admission must wait
    server = Server(budget)
    tickets = []
    for sc, steps in reqs:
        tickets.append(server.submit(sc.parameters, sc.positions, boundary_of(sc), sc.refinement, sc.dt, steps,
                                     sc.refinement.max_particle_count if sc.refinement else None))
    seen_queue = False
    while True:
        left = server.poll(7)
        st = server.stats()
        assert st["used_bytes"] <= budget
        seen_queue |= st["queued"] > 0
        if left == 0:
            break
    assert seen_queue, "the budget must make requests wait"
    for (sc, steps), t in zip(reqs, tickets):
        s = server.status(t)
        assert s["state"] == "done" and s["steps_done"] == steps
        assert s["submit_s"] <= s["admit_s"] <= s["finish_s"]
        got = server.take(t)
        want = _alone(sc, steps)
        for k in ("ids", "positions", "velocities", "densities", "radii"):
            assert_bitexact(k, got[k], want[k])
    server.close()


def test_server_queue_and_budget_on_the_host():
    """Host-only part of the server (no GPU): requests that could never fit are refused, the others queue in order
    with their memory estimate."""
    from adaptivesph_gb300 import AsphError

    sc = small_dam_break()
    need = _bytes(sc)
    server = Server(need // 2)
    with pytest.raises(AsphError):
        server.submit(sc.parameters, sc.positions, boundary_of(sc), None, sc.dt, 5)
    server.close()
    server = Server(3 * need)
    t1 = server.submit(sc.parameters, sc.positions, boundary_of(sc), None, sc.dt, 5)
    t2 = server.submit(sc.parameters, sc.positions, boundary_of(sc), None, sc.dt, 7)
    for t, steps in ((t1, 5), (t2, 7)):
        s = server.status(t)
        assert s["state"] == "queued" and s["steps"] == steps and s["device_bytes"] == need
    assert server.stats()["queued"] == 2
    server.close()


@pytest.mark.gpu
def test_estimate_matches_device_memory():
    """The estimate is the figure at the fluid capacity; at creation the neighbour rows (128 entries of 8 bytes per
    particle) are allocated for n + n/8 + 256 particles (in multiples of 256), the rest of the capacity's rows only
    when a step needs them."""
    torch = pytest.importorskip("torch")
    sc = small_dam_break(counts=(40, 40, 40), refinement=adaptive_refinement(capacity=300000))
    bd = boundary_of(sc)
    est = _bytes(sc)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd, sc.refinement, 300000,
                            bd.get_particle_count())
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert sim.device_bytes() == est
    used = free0 - free1
    n, cap = sc.positions.shape[0], 300000
    rows = min(cap, (n + n // 8 + 256 + 255) // 256 * 256)
    now = est - (cap - rows) * 128 * 8
    assert abs(used - now) <= 0.05 * now + (64 << 20), (used, now, est)
    sim.close()


@pytest.mark.gpu
def test_server_requests_arriving_while_polling_equal_alone():
    """Continuous batching: a second thread submits requests one by one while the main thread polls (so requests
    arrive while others are on the GPU and are admitted as memory frees up); every result equals the request run
    alone, bit for bit, and the budget holds throughout."""
    import threading
    import time

    # the first request runs long enough (400 steps) that the others arrive while it is on the GPU
    reqs = [(small_dam_break(counts=(12, 24, 12), seed=21), 400)] + _requests() + [
        (small_dam_break(counts=(9, 14, 9), seed=12, refinement=adaptive_refinement()), 33),
        (small_dam_break(counts=(7, 9, 7), seed=13), 20)]
    sizes = [_bytes(sc) for sc, _ in reqs]
    budget = int(sum(sorted(sizes)[-3:]) * 1.01)  # room for about three requests at a time
    server = Server(budget)
    tickets = [None] * len(reqs)
    first_admitted = threading.Event()
    submitted_all = threading.Event()
    errors = []
    arrived_while_running = [0]

    def submitter():
        try:
            for k, (sc, steps) in enumerate(reqs):
                if server.stats()["active"] > 0:
                    arrived_while_running[0] += 1
                tickets[k] = server.submit(sc.parameters, sc.positions, boundary_of(sc), sc.refinement, sc.dt, steps,
                                           sc.refinement.max_particle_count if sc.refinement else None)
                if k == 0:
                    first_admitted.wait(timeout=60)  # the rest arrive once the first one runs
                time.sleep(0.002)
        except Exception as e:  # surfaced by the main thread
            errors.append(e)
        finally:
            submitted_all.set()

    th = threading.Thread(target=submitter)
    th.start()
    polls = 0
    while True:
        if server.stats()["active"] > 0:
            first_admitted.set()
        left = server.poll(3)
        polls += 1
        assert server.stats()["used_bytes"] <= budget
        if left == 0 and submitted_all.is_set() and all(t is not None for t in tickets):
            if server.poll(1) == 0:
                break
        if left == 0:
            time.sleep(0.005)
        assert polls < 100000
    th.join()
    assert not errors, errors
    assert arrived_while_running[0] >= 3, "requests must arrive while others are running"
    for (sc, steps), t in zip(reqs, tickets):
        s = server.status(t)
        assert s["state"] == "done" and s["steps_done"] == steps
        got = server.take(t)
        want = _alone(sc, steps)
        for k in ("ids", "positions", "velocities", "densities", "radii"):
            assert_bitexact(k, got[k], want[k])
    server.close()
