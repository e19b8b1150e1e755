"""Benchmark: particle-steps/s of the adaptive 1M-particle dam break on one GB300 (per GPU, replicas for N > 1).

Workload (the configuration the headline metric is quoted on): 100x200x50 = 1,000,000 particles at dx = 0.004 m,
+-0.05 dx jitter (seed 2), in a 1.6 x 1.0 x 0.67 m tank with ~503k wall particles, Tait c0 = 10 sqrt(2 g 0.8),
h = 1.3 dx, artificial viscosity 0.01, fixed dt = 0.25 h / c0, Vacondio refinement (velocity criterion,
minMassRatio 0.05, maxMassRatio 8, capacity 4M, batch ratio 0.2, cooldowns 10/10). Synthetic seeded data.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line from rank 0. `value` times K steps with the state resident in HBM (CUDA events on the simulation's
stream, barrier + synchronize on both sides, max over ranks). `e2e` times the same steps through the public C ABI
with host buffers: the simulation is created from host positions inside the timed region and every step's result
(positions, velocities, densities, radii) is exported to pinned host memory. `late` continues the simulation to
frame 150 and times 20 frames there. `--impl reference` times the reference algorithm as the oracle's FP64 step
on all host cores (the reference itself has no CPU path) over the same frames, without loading the CUDA library.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

# many simulations step on their own streams in the batched workload: let them use all 32 hardware queues
# (the default of 8 makes unrelated streams wait on one another); set before CUDA is initialised
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 1M (adaptive dam break)"
UNIT = "particle-steps/s"
WORKLOAD = "adaptive dam break, 1M particles (100x200x50, dx=0.004 m), cap 4M, velocity criterion"
# algorithmic HBM bytes per particle of the density pass (the step's dominant kernel): read x, h, m; write rho
DENSITY_BYTES_PER_PARTICLE = 28.0
# algorithmic HBM bytes per particle-step of the whole step (integrate 80, keys 24, 3 sort passes 48,
# cell tables 4, reorder 88, density 28, force 60)
STEP_BYTES_PER_PARTICLE = 332.0
L2_BYTES = 129e6
LATE_STEPS = 20  # frames timed by the late-frame leg
PLAIN_WARMUP = 20  # untimed frames before the plain legs (ours and the reference's CUDA step)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_density():
    """DRAM bytes per particle and pipe utilisation of one density launch from the committed ncu record, if
    present (an empty dict otherwise)."""
    p = os.path.join(ROOT, "profiles", "density_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


# ------------------------------------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------------ scene
def c2_scene(args):
    from adaptivesph_gb300 import scenes
    from adaptivesph_gb300.parameters import Criterion

    return scenes.c2_adaptive(criterion=Criterion.FREE_SURFACE if args.criterion == "free_surface"
                              else Criterion.VELOCITY)


def build_scene(args):
    from adaptivesph_gb300 import StaticBoundaryDomain

    sc = c2_scene(args)
    bd = StaticBoundaryDomain.generate(sc.parameters.domain, sc.boundary_spacing, sc.parameters.rest_density,
                                       sc.parameters.base_smoothing_radius)
    return sc, bd


def build_scene_cpu(args):
    """The same scene for the CPU legs: the seeded lattice (pure numpy) and walls from the oracle's restatement of
    StaticBoundaryDomain::generate, so that the CUDA library is never loaded (bit-identical walls: the parity
    tests compare both generators)."""
    import oracle

    sc = c2_scene(args)
    d = sc.parameters.domain
    pos, psi = oracle.boundary_generate(d.min, d.max, sc.boundary_spacing, sc.parameters.rest_density,
                                        sc.parameters.base_smoothing_radius)
    return sc, pos, psi


def workload_config(sc, nb: int, world: int, args) -> dict:
    """The workload as both arms report it (identical dicts)."""
    n0 = int(sc.positions.shape[0])
    workload = WORKLOAD if args.criterion == "velocity" else WORKLOAD.replace("velocity criterion",
                                                                             "free-surface criterion")
    return {
        "workload": workload,
        "particles_initial": n0,
        "boundary_particles": nb,
        "capacity": int(sc.refinement.max_particle_count),
        "dt": sc.dt,
        "l2": f"inputs larger than L2: ~{device_state_bytes(sc.refinement.max_particle_count, n0, nb) / 1e6:.0f} MB "
              f"of device state touched per step vs {L2_BYTES / 1e6:.0f} MB L2; no flush",
        "parallelism": f"replicas x{world}",
    }


def device_state_bytes(n_cap: int, n: int, nb: int) -> int:
    # two buffer sets of (ph, vm, acc, rp, rad, id) + kernel constants + sort buffers, per particle
    return n * (2 * 64 + 16 + 16) + nb * 24


# ------------------------------------------------------------------------------------------------ CPU leg
def cpu_throughput(args, steps: int, warmup: int):
    """The oracle's FP64 step (the reference algorithm restated on the CPU, double precision throughout) on the same
    workload, all host threads: `warmup` untimed steps, then `steps` timed ones. Returns (particle-steps/s, threads,
    seconds, frames timed)."""
    import oracle

    sc, bpos, bpsi = build_scene_cpu(args)
    o = oracle.OracleSim64(sc.parameters, sc.positions, bpos, bpsi, sc.refinement,
                           capacity=sc.refinement.max_particle_count)
    for _ in range(warmup):
        o.step(sc.dt)
    ps = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        ps += o.n
        o.step(sc.dt)
    dt = time.perf_counter() - t0
    return ps / dt, oracle.get_threads(), dt, (warmup, warmup + steps - 1)


# ------------------------------------------------------------------------------------------------ replicas
def gather_rows(local, dist, world: int, device: str) -> np.ndarray:
    """Every rank's [particle-steps, seconds, e2e particle-steps, e2e seconds], one row per rank."""
    import torch

    t = torch.tensor(local, dtype=torch.float64, device=device)
    gathered = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(gathered, t)
    return torch.stack(gathered).cpu().numpy()


def replica_throughput(rows: np.ndarray):
    """Whole-job throughput of independent replicas: the work of all ranks over the slowest rank's time (device
    timed and end to end)."""
    value = float(rows[:, 0].sum()) / float(rows[:, 1].max())
    e2e_time = float(rows[:, 3].max())
    e2e = float(rows[:, 2].sum()) / e2e_time if e2e_time > 0 else 0.0
    return value, e2e


# ------------------------------------------------------------------------------------------------ GPU leg
def run_ours(args, rank: int, world: int, dist):
    import torch

    from adaptivesph_gb300 import create_simulation

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    sc, bd = build_scene(args)
    n0 = sc.positions.shape[0]
    if args.capacity:
        sc.refinement.max_particle_count = args.capacity
    cap = sc.refinement.max_particle_count
    stream = torch.cuda.Stream()

    # ---------------- device-resident throughput
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd, sc.refinement, cap, bd.get_particle_count())
    sim.set_stream(stream.cuda_stream)
    for _ in range(args.warmup):
        sim.step_async(sc.dt)
    sim.synchronize()
    counts = []
    sim.enable_timing(True)
    launches0 = sim.launch_count()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(dev)
    sampler.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        torch.cuda.nvtx.range_push("timed")  # NVTX ranges let a profiler capture just these frames
        start.record(stream)
        for _ in range(args.steps):
            counts.append(sim.get_fluid_particles_count())
            sim.step_async(sc.dt)
        end.record(stream)
        torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    sim.synchronize()
    ms = start.elapsed_time(end)
    launches = sim.launch_count() - launches0
    kt = sim.kernel_times()
    sim.enable_timing(False)
    particle_steps = float(sum(counts))
    errors = sim.device_errors()
    n_end = sim.get_fluid_particles_count()
    frame_end = args.warmup + args.steps

    # ---------------- late frames: the same simulation continued, untimed, to frame --late-frame (merged particles of
    # several h0 exist from about frame 100 on), then LATE_STEPS frames timed like the main leg
    late = None
    if not args.no_late and frame_end <= args.late_frame:
        for _ in range(args.late_frame - frame_end):
            sim.step_async(sc.dt)
        sim.synchronize()
        sim.enable_timing(True)
        late_counts = []
        ls, le = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            torch.cuda.nvtx.range_push("late")
            ls.record(stream)
            for _ in range(LATE_STEPS):
                late_counts.append(sim.get_fluid_particles_count())
                sim.step_async(sc.dt)
            le.record(stream)
            torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        late_ms = ls.elapsed_time(le)
        lkt = sim.kernel_times()
        sim.enable_timing(False)
        late = {"value": float(sum(late_counts)) / (late_ms / 1e3), "unit": UNIT,
                "ms_per_step": late_ms / LATE_STEPS, "frames": [args.late_frame, args.late_frame + LATE_STEPS - 1],
                "particles": [late_counts[0], sim.get_fluid_particles_count()],
                "kernel_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in lkt.items()},
                "what": f"the same simulation continued untimed to frame {args.late_frame}, then {LATE_STEPS} frames "
                        "timed with the state resident (CUDA events on the simulation's stream); merged particles "
                        "of several h0 make the later frames of the 2000-step run slower"}
        errors |= sim.device_errors()
    sim.close()

    # ---------------- plain form: the same 1M scene without refinement, frames PLAIN_WARMUP .. PLAIN_WARMUP + K - 1
    # from the lattice, timed like the main leg; the reference arm times the reference's own CUDA step on the same
    # frames (its GPU leg), so the two plain numbers compare like for like
    plain = None
    if args.plain_steps > 0:
        simp = create_simulation(sc.parameters, sc.positions, None, None, bd, None, n0, bd.get_particle_count())
        simp.set_stream(stream.cuda_stream)
        for _ in range(PLAIN_WARMUP):
            simp.step_async(sc.dt)
        simp.synchronize()
        ps, pe = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ps.record(stream)
            for _ in range(args.plain_steps):
                simp.step_async(sc.dt)
            pe.record(stream)
        torch.cuda.synchronize()
        plain_ms = ps.elapsed_time(pe)
        errors |= simp.device_errors()
        plain = {"value": n0 * args.plain_steps / (plain_ms / 1e3), "unit": UNIT,
                 "ms_per_step": plain_ms / args.plain_steps, "steps": args.plain_steps,
                 "frames": [PLAIN_WARMUP, PLAIN_WARMUP + args.plain_steps - 1], "particles": n0,
                 "what": "the same 1M-particle dam break and walls without refinement (the reference's plain "
                         "SphSimulation step), state resident, CUDA events on the simulation's stream"}
        simp.close()
        # the 128k plain dam break (40x80x40 at dx 0.01 m), the same way
        from adaptivesph_gb300 import StaticBoundaryDomain, scenes as _scenes

        c1 = _scenes.c1_plain()
        bd1 = StaticBoundaryDomain.generate(c1.parameters.domain, c1.boundary_spacing, c1.parameters.rest_density,
                                            c1.parameters.base_smoothing_radius)
        n1 = c1.positions.shape[0]
        sim1 = create_simulation(c1.parameters, c1.positions, None, None, bd1, None, n1, bd1.get_particle_count())
        sim1.set_stream(stream.cuda_stream)
        for _ in range(PLAIN_WARMUP):
            sim1.step_async(c1.dt)
        sim1.synchronize()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ps.record(stream)
            for _ in range(args.plain_steps):
                sim1.step_async(c1.dt)
            pe.record(stream)
        torch.cuda.synchronize()
        c1_ms = ps.elapsed_time(pe)
        errors |= sim1.device_errors()
        plain["c1_128k"] = {"value": n1 * args.plain_steps / (c1_ms / 1e3), "unit": UNIT,
                            "ms_per_step": c1_ms / args.plain_steps, "particles": n1,
                            "boundary_particles": bd1.get_particle_count(),
                            "what": "the 128k plain dam break (40x80x40, dx 0.01 m), frames "
                                    f"{PLAIN_WARMUP}..{PLAIN_WARMUP + args.plain_steps - 1}"}
        sim1.close()

    # ---------------- end to end through the C ABI with host buffers: the simulation is created from host arrays
    # inside the timed region and every frame's result is exported to pinned host memory; it covers frames
    # 0 .. warmup + steps - 1 (the device-resident run times frames warmup .. warmup + steps - 1)
    e2e_counts = []
    d2h = 0
    e2e_s = 0.0
    create_s = 0.0
    h2d = 0.0
    if not args.no_e2e:
        torch.cuda.synchronize()
        # two sets of pinned host arrays: frame k is copied into set k % 2 while frame k + 1 is computed
        pinned = [{
            "positions": torch.empty((cap, 4), dtype=torch.float32, pin_memory=True).numpy(),
            "velocities": torch.empty((cap, 4), dtype=torch.float32, pin_memory=True).numpy(),
            "densities": torch.empty((cap,), dtype=torch.float32, pin_memory=True).numpy(),
            "radii": torch.empty((cap,), dtype=torch.float32, pin_memory=True).numpy(),
        } for _ in range(2)]
        t0 = time.perf_counter()
        sim2 = create_simulation(sc.parameters, sc.positions, None, None, bd, sc.refinement, cap,
                                 bd.get_particle_count())
        create_s = time.perf_counter() - t0
        for k in range(args.warmup + args.steps):
            n_now = sim2.get_fluid_particles_count()
            sim2.step_async(sc.dt)
            sim2.export_wait()  # frame k - 1 is on the host now, while frame k computes
            out = {key: v[:sim2.get_fluid_particles_count()] for key, v in pinned[k % 2].items()}
            sim2.export_host_async(out)
            e2e_counts.append(n_now)
            d2h += sum(v.nbytes for v in out.values())
        sim2.export_wait()
        e2e_s = time.perf_counter() - t0
        sim2.close()
        h2d = (n0 * 16 + bd.get_particle_count() * 20) / len(e2e_counts)

    local = [particle_steps, ms / 1e3, float(sum(e2e_counts)), e2e_s]
    rows = gather_rows(local, dist, world, "cuda") if dist is not None else np.array([local])
    value, e2e_total = replica_throughput(rows)
    if rank != 0:
        return None

    d_ms, d_launches = kt["density"]
    avg_density_ms = d_ms / max(d_launches, 1)
    mean_n = particle_steps / max(args.steps, 1)
    peak, peak_kind = measured_peaks()
    achieved = DENSITY_BYTES_PER_PARTICLE * mean_n / (avg_density_ms * 1e-3) / 1e9
    prof = profiled_density()
    traffic_pp = prof.get("dram_bytes_per_particle")
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": float(rows[:, 1].max()) * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded lattice + jitter; no dataset involved)",
        "config": workload_config(sc, bd.get_particle_count(), world, args),
        "frames_timed": [args.warmup, frame_end - 1],
        "particles_final": n_end,
        "refinement_frames_timed": sum(1 for f in range(args.warmup, frame_end) if f == 10 or (f > 10 and f % 10 == 0)),
        "roofline": {
            "bound": "hbm",
            "kernel": "density pass (k_density with its heavy and long-row kernels)",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": None if traffic_pp is None else traffic_pp * mean_n,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "algorithmic_bytes_per_particle": DENSITY_BYTES_PER_PARTICLE,
            "avg_launch_ms": avg_density_ms,
            "traffic_source": prof.get("source"),
            "limiter": "instruction issue",
            "issue": {"issue_slots_busy": prof.get("issue_slots_busy"), "fma_pipe": prof.get("fma_pipe"),
                      "alu_pipe": prof.get("alu_pipe"), "dram_throughput": prof.get("dram_throughput"),
                      "source": "the same ncu capture as traffic"},
            "note": "the density pass is bound by instruction issue in its candidate scan (issue slots and the "
                    "FMA/ALU pipes above, a few % of DRAM peak), not by HBM; the HBM fraction is small by "
                    "construction (28 algorithmic bytes per particle against ~1 us of scan work)",
        },
        "step_roofline": {
            "achieved": STEP_BYTES_PER_PARTICLE * value / 1e9,
            "unit": "GB/s",
            "frac": STEP_BYTES_PER_PARTICLE * value / 1e9 / peak,
            "algorithmic_bytes_per_particle_step": STEP_BYTES_PER_PARTICLE,
        },
        "kernel_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in kt.items()},
        "e2e": {"value": e2e_total, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h / max(len(e2e_counts), 1), "steps": len(e2e_counts),
                "create_ms": create_s * 1e3, "total_ms": e2e_s * 1e3,
                "includes": "create from host positions, then every frame a step and an asynchronous export to "
                            "pinned host memory (frame k is copied while frame k+1 computes), frames "
                            "0..warmup+steps-1, timed until the last frame is on the host"},
        "gpu_launches": int(launches),
        "device_errors": errors,
        "clocks": clocks,
    }
    if late is not None:
        line["late"] = late
    if plain is not None:
        line["plain"] = plain
    if not args.no_cpu:
        cps, cores, secs, (f0, f1) = cpu_throughput(args, args.cpu_steps, 1)
        line["cpu_baseline"] = {"value": cps, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"the oracle's FP64 step: {args.cpu_steps} steps of the same 1M-particle "
                                          f"workload after 1 warm-up step (frames {f0}..{f1}, refinement at frame 10), "
                                          f"{secs:.1f} s"}
    return line


def run_reference(args, rank: int, world: int):
    """The reference arm: the reference has no CPU path and no published number, and its CUDA library is not part of
    this arm; the algorithm runs as the oracle's FP64 step (a restatement of the reference's step, double precision
    throughout) on all host cores, over the same frames as the GPU arm (`warmup` untimed, then `steps` timed, at
    most --ref-steps of them). The CUDA library of this repository is never loaded here."""
    if rank != 0:
        return None
    import adaptivesph_gb300._lib as product_lib

    steps = min(args.steps, args.ref_steps)
    sc, bpos, bpsi = build_scene_cpu(args)
    cps, cores, secs, (f0, f1) = cpu_throughput(args, steps, args.warmup)
    ref_gpu = reference_cuda_leg(args, sc, bpos, bpsi) if args.plain_steps > 0 else None
    if ref_gpu is not None and "unavailable" not in ref_gpu:
        import oracle
        from adaptivesph_gb300 import scenes as _scenes

        c1 = _scenes.c1_plain()
        d1 = c1.parameters.domain
        bp1, bs1 = oracle.boundary_generate(d1.min, d1.max, c1.boundary_spacing, c1.parameters.rest_density,
                                            c1.parameters.base_smoothing_radius)
        ref_gpu["c1_128k"] = reference_cuda_leg(args, c1, bp1, bs1)
        ref_gpu["c1_128k"]["what"] = "the same, on the 128k plain dam break (40x80x40, dx 0.01 m)"
        ref_gpu["c1_128k"].pop("clocks", None)
    if product_lib._lib is not None:
        raise RuntimeError("the reference arm must not load the CUDA library")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": cps,
        "unit": UNIT,
        "n_gpus": world,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": secs / steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded lattice + jitter; no dataset involved)",
        "config": workload_config(sc, int(bpos.shape[0]), world, args),
        "frames_timed": [f0, f1],
        "cpu_baseline": {"value": cps, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"frames {f0}..{f1} of the 1M-particle workload ({steps} steps after {args.warmup} "
                                   f"untimed), {secs:.1f} s: the oracle's FP64 step (the reference has no CPU path)"},
        "e2e": {"value": cps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if ref_gpu is not None:
        line["reference_cuda"] = ref_gpu
    return line


def reference_cuda_leg(args, sc, bpos, bpsi):
    """The reference's own CUDA step on this GPU (oracle/ref_cuda.py: its kernels compiled from its sources for
    sm_103a, launched in SphSimulation::update's order with its block size and its device synchronisation after
    every step) on the plain form of a scene (the 1M-particle dam break, and the 128k one beside it), frames
    PLAIN_WARMUP .. PLAIN_WARMUP + K - 1: what the GPU arm's `plain` leg is compared with. The reference's
    refinement pass is not run on the GPU (its in-place compaction races)."""
    from oracle import ref_cuda

    if not ref_cuda.available():
        return {"unavailable": "the reference's kernels are built into oracle/_ref where the reference checkout is "
                               "present, and none were found"}
    import torch

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    r = ref_cuda.RefCudaSim(sc.parameters, sc.positions, bpos, bpsi)
    for _ in range(PLAIN_WARMUP):
        r.step(sc.dt)
    steps = args.plain_steps
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    sampler = ClockSampler(dev)
    sampler.start()
    torch.cuda.synchronize()
    s.record()
    marks[0].record()
    for k in range(steps):
        r.step(sc.dt)  # ends with the device synchronisation the reference's update() ends with
        marks[k + 1].record()
    e.record()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = s.elapsed_time(e)
    per_step = sorted(marks[k].elapsed_time(marks[k + 1]) for k in range(steps))
    n = r.n
    rho = r.rho[:n].float()
    ok = bool(torch.isfinite(rho).all().item())
    r.close()
    return {"value": n * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
            "ms_per_step_median": per_step[len(per_step) // 2], "steps": steps,
            "frames": [PLAIN_WARMUP, PLAIN_WARMUP + steps - 1], "particles": n, "boundary_particles": int(bpos.shape[0]),
            "densities_finite": ok, "clocks": clocks,
            "what": "the reference's own kernels (cubins built from its sources, C++20, --expt-relaxed-constexpr, "
                    "ptxas -O3, default FMA contraction) run in SphSimulation::update's order on the plain form of "
                    "the 1M-particle dam break (no refinement), 256-thread blocks, a device synchronisation after "
                    "every step; thrust::sort_by_key of the cell indices replaced by torch.sort (both CUB radix "
                    "sorts); CUDA events around the timed steps"}


# ------------------------------------------------------------------------------------------------ batched mix
def run_batched(args, rank: int, world: int, dist):
    """The 256-scene mix (scenes.batched_mix): every scene advanced together through asph_batch_step, against the
    same scenes advanced one after another, each step through asph_simulation_update (sequential plain)."""
    import torch

    from adaptivesph_gb300 import Batch, StaticBoundaryDomain, create_simulation, scenes

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    mix = scenes.batched_mix(count=args.scenes)
    sims = []
    t0 = time.perf_counter()
    for sc in mix:
        bd = StaticBoundaryDomain.generate(sc.parameters.domain, sc.boundary_spacing, sc.parameters.rest_density,
                                           sc.parameters.base_smoothing_radius)
        cap = sc.refinement.max_particle_count if sc.refinement else sc.positions.shape[0]
        sims.append(create_simulation(sc.parameters, sc.positions, None, None, bd, sc.refinement, cap,
                                      bd.get_particle_count()))
    setup_s = time.perf_counter() - t0
    dts = [sc.dt for sc in mix]
    batch = Batch(sims)  # mode "auto": the autotuner times its candidates over the first plain frames
    tune_steps = 0
    while not batch.tuning()["tuned"] and tune_steps < 200:
        batch.step(dts, 5)
        tune_steps += 5
    batch.step(dts, args.warmup)

    # each mode over the same number of frames, continuing the same simulations (results are identical in every
    # mode; only the time differs)
    modes = {}
    mode_steps = min(args.steps, 100)
    for mode in ("graphs", "segmented", "auto"):
        batch.set_mode(mode)
        batch.step(dts, 3)  # captures
        nb = [s.get_fluid_particles_count() for s in sims]
        torch.cuda.synchronize()
        tm = time.perf_counter()
        batch.step(dts, mode_steps)
        torch.cuda.synchronize()
        el = time.perf_counter() - tm
        na = [s.get_fluid_particles_count() for s in sims]
        modes[mode] = {"value": float(sum(0.5 * (a + b) for a, b in zip(nb, na))) * mode_steps / el,
                       "ms_per_step": el * 1e3 / mode_steps, "steps": mode_steps}
    n_before = [s.get_fluid_particles_count() for s in sims]
    if dist is not None:
        dist.barrier()
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch.step(dts, args.steps)
    torch.cuda.synchronize()
    batched_s = time.perf_counter() - t0
    clocks = sampler.stop()
    n_after = [s.get_fluid_particles_count() for s in sims]
    work = float(sum(0.5 * (a + b) for a, b in zip(n_before, n_after))) * args.steps
    stats = batch.stats()
    tuning = batch.tuning()
    batch.close()
    # sequential: the same simulations, continuing, one scene at a time
    seq_work, seq_s, per_scene = 0.0, 0.0, []
    for s, dt in zip(sims, dts):
        n0 = s.get_fluid_particles_count()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(args.steps):
            s.update(dt)
        e = time.perf_counter() - t
        seq_s += e
        seq_work += 0.5 * (n0 + s.get_fluid_particles_count()) * args.steps
        per_scene.append(e / args.steps * 1e3)
    for s in sims:
        s.close()
    rows = np.array([[work, batched_s, seq_work, seq_s]])
    if dist is not None:
        rows = gather_rows(rows[0].tolist(), dist, world, "cuda")
    if rank != 0:
        return None
    value = float(rows[:, 0].sum()) / float(rows[:, 1].max())
    seq = float(rows[:, 2].sum()) / float(rows[:, 3].sum())
    ps = np.array(per_scene)
    return {
        "metric": "particle-steps/s, batched scene mix",
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": batched_s * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded scene mix; no dataset involved)",
        "config": {"workload": f"{len(mix)} dam-break scenes, particles log-uniform 4k-256k "
                               f"({sum(sc.positions.shape[0] for sc in mix)} in total), fill U(0.2, 0.6), Morris nu "
                               f"log-uniform 1e-6..1e-3, refinement on even scenes",
                   "parallelism": f"replicas x{world}", "setup_s": setup_s},
        "scene_steps_per_s": len(mix) * args.steps / float(rows[:, 1].max()),
        "sequential": {"value": seq, "unit": UNIT,
                       "what": "the same scenes one after another, asph_simulation_update per step",
                       "ms_per_step_p50": float(np.percentile(ps, 50)), "ms_per_step_p99": float(np.percentile(ps, 99))},
        "speedup_vs_sequential": value / seq,
        "batch": stats,
        "tuning": tuning,
        "tuning_steps": tune_steps,
        "modes": modes,
        "clocks": clocks,
    }


def run_batch_one(args, rank: int, world: int, dist):
    """The 1M-particle dam break without refinement, alone in an asph_batch in mode --batch-mode: 8 frames untimed,
    then --steps frames timed inside the NVTX range "timed" (a profiler's capture window). Compares the segmented
    passes with per-simulation graphs on the same particles."""
    import torch

    from adaptivesph_gb300 import Batch, create_simulation

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    sc, bd = build_scene(args)
    sc.refinement = None
    n0 = sc.positions.shape[0]
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd, None, n0, bd.get_particle_count())
    batch = Batch([sim], mode=args.batch_mode)
    batch.step([sc.dt], 8)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("timed")
    batch.step([sc.dt], args.steps)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    tuning = batch.tuning()
    batch.close()
    sim.close()
    if rank != 0:
        return None
    return {"metric": "particle-steps/s, one scene in a batch", "value": n0 * args.steps / el, "unit": UNIT,
            "ms_per_step": el * 1e3 / args.steps, "steps": args.steps, "batch_mode": args.batch_mode,
            "segmented_steps": tuning["segmented_steps"],
            "config": {"workload": "1M-particle dam break (100x200x50, dx 0.004 m) without refinement, alone in a batch"}}


# ------------------------------------------------------------------------------------------------ served
def _pct(v, q):
    return float(np.percentile(np.asarray(v, np.float64), q)) if len(v) else None


def run_served(args, rank: int, world: int, dist):
    """Scene requests (scenes.served_requests) arriving as a Poisson stream at each rate of --rates, served by
    asph_server (continuous batching under a device-memory budget), against the same requests run one at a time in
    arrival order (first come first served, each alone through asph_simulation_update); latency = finish - arrival."""
    import torch

    from adaptivesph_gb300 import Server, StaticBoundaryDomain, create_simulation_with_walls, scenes

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    reqs = scenes.served_requests(count=args.requests)
    # wall generation per request: the host generator against the GPU one (the served path uses the GPU one at
    # admission, the requests carry only their parameters and fluid positions)
    host_walls_s, gpu_walls_s, wall_counts = [], [], []
    for sc, _ in reqs:
        wargs = (sc.parameters.domain, sc.boundary_spacing, sc.parameters.rest_density,
                 sc.parameters.base_smoothing_radius)
        t = time.perf_counter()
        bd = StaticBoundaryDomain.generate(*wargs)
        host_walls_s.append(time.perf_counter() - t)
        torch.cuda.synchronize()
        t = time.perf_counter()
        StaticBoundaryDomain.generate(*wargs, device=True)
        gpu_walls_s.append(time.perf_counter() - t)
        wall_counts.append(bd.get_particle_count())
    work = float(sum(sc.positions.shape[0] * steps for sc, steps in reqs))
    budget = int(args.budget_gb * 1e9)
    # sequential: every request alone (walls generated on the GPU), its service time measured; queueing follows from
    # the arrival times
    service = []
    for sc, steps in reqs:
        cap = sc.refinement.max_particle_count if sc.refinement else sc.positions.shape[0]
        torch.cuda.synchronize()
        t = time.perf_counter()
        sim = create_simulation_with_walls(sc.parameters, sc.positions, sc.boundary_spacing, sc.refinement, cap)
        for _ in range(steps):
            sim.update(sc.dt)
        sim.export_host()
        service.append(time.perf_counter() - t)
        sim.close()
    rng = np.random.default_rng(5)
    results = []
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    for rate in args.rates:
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=len(reqs)))
        # sequential first come first served
        t_free, seq_lat = 0.0, []
        for a, s in zip(arrivals, service):
            start = max(a, t_free)
            t_free = start + s
            seq_lat.append(t_free - a)
        seq_makespan = t_free
        # served
        server = Server(budget)
        t0 = time.perf_counter()  # the server's clock starts with it: arrival times are on the same clock
        tickets, nxt = [], 0
        while True:
            now = time.perf_counter() - t0
            while nxt < len(reqs) and arrivals[nxt] <= now:
                sc, steps = reqs[nxt]
                tickets.append(server.submit(sc.parameters, sc.positions, None, sc.refinement, sc.dt, steps,
                                             sc.refinement.max_particle_count if sc.refinement else None,
                                             wall_spacing=sc.boundary_spacing))
                nxt += 1
            left = server.poll(args.poll_steps)
            if left == 0:
                if nxt == len(reqs):
                    break
                time.sleep(max(0.0, min(0.01, arrivals[nxt] - (time.perf_counter() - t0))))
        lat, finish = [], []
        for k, t in enumerate(tickets):
            st = server.status(t)
            assert st["state"] == "done", st
            lat.append(st["finish_s"] - arrivals[k])
            finish.append(st["finish_s"])
            server.take(t)
        stats = server.stats()
        server.close()
        makespan = max(finish)
        results.append({
            "rate_per_s": rate,
            "served": {"scenes_per_s": len(reqs) / makespan, "particle_steps_per_s": work / makespan,
                       "latency_s": {"p50": _pct(lat, 50), "p95": _pct(lat, 95), "p99": _pct(lat, 99)},
                       "graph_steps": stats["graph_steps"], "eager_steps": stats["eager_steps"]},
            "sequential": {"scenes_per_s": len(reqs) / seq_makespan, "particle_steps_per_s": work / seq_makespan,
                           "latency_s": {"p50": _pct(seq_lat, 50), "p95": _pct(seq_lat, 95),
                                         "p99": _pct(seq_lat, 99)}},
        })
    clocks = sampler.stop()
    if rank != 0:
        return None
    best = max(r["served"]["particle_steps_per_s"] for r in results)
    seq_best = max(r["sequential"]["particle_steps_per_s"] for r in results)
    return {
        "metric": "particle-steps/s, served scene requests",
        "value": best,
        "unit": UNIT,
        "n_gpus": world,
        "steps": int(sum(s for _, s in reqs)),
        "warmup": 0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded requests and Poisson arrivals; no dataset involved)",
        "config": {"workload": f"{len(reqs)} dam-break requests, 8k-1M particles (log-uniform), refinement p=0.5, "
                               f"200-2000 steps, Poisson arrivals", "budget_bytes": budget,
                   "poll_steps": args.poll_steps, "parallelism": f"replicas x{world}"},
        "speedup_vs_sequential": best / seq_best,
        "rates": results,
        "walls_per_request": {"particles_mean": float(np.mean(wall_counts)),
                              "host_s_mean": float(np.mean(host_walls_s)), "gpu_s_mean": float(np.mean(gpu_walls_s)),
                              "what": "StaticBoundaryDomain::generate per request: host threads against the GPU "
                                      "kernels (bit-identical walls); the served and sequential runs use the GPU"},
        "clocks": clocks,
    }


# ------------------------------------------------------------------------------------------------ conservation
def _totals_row(sim, frame):
    t = sim.totals()
    return {"frame": frame, "count": t["count"], "mass": t["mass"], "momentum": list(t["momentum"]),
            "kinetic_energy": t["kinetic_energy"]}


def _conservation_run(sc, steps, every, adaptive):
    """FP64 totals of one simulation every `every` steps over `steps` steps, with the refinement reports."""
    import torch

    from adaptivesph_gb300 import StaticBoundaryDomain, create_simulation

    if sc.boundary_spacing > 0:
        bd = StaticBoundaryDomain.generate(sc.parameters.domain, sc.boundary_spacing, sc.parameters.rest_density,
                                           sc.parameters.base_smoothing_radius, device=True)
    else:
        bd = StaticBoundaryDomain.empty(sc.parameters.domain)
    n0 = sc.positions.shape[0]
    cap = sc.refinement.max_particle_count if adaptive else n0
    sim = create_simulation(sc.parameters, sc.positions, None, None, bd, sc.refinement if adaptive else None, cap,
                            max(bd.get_particle_count(), 1))
    if sc.velocities is not None:
        st = sim.read_state()
        st["vel"] = sc.velocities.copy()
        sim.write_state(st, next_id=n0)
    rows = [_totals_row(sim, 0)]
    refinements = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rows[0]["seconds"] = 0.0
    for k in range(1, steps + 1):
        sim.step_async(sc.dt)
        if k % every == 0 or k == steps:
            rows.append(_totals_row(sim, k))  # the totals read drains the stream: the time is the steps' own
            rows[-1]["seconds"] = time.perf_counter() - t0
        if adaptive and (k - 1 == sc.refinement.initial_cooldown or
                         (k - 1 > sc.refinement.initial_cooldown and (k - 1) % sc.refinement.cooldown == 0)):
            r = sim.last_refinement()
            refinements.append({"frame": r["frame"], "merge_pairs": r["merge_pairs"], "splits": r["splits"],
                                "count_after": r["count_after"]})
    sim.synchronize()
    secs = time.perf_counter() - t0
    errors = sim.device_errors()
    sim.close()
    return rows, refinements, secs, errors


def _drift_summary(rows, refinements, sc, every):
    m0 = rows[0]["mass"]
    P0 = np.array(rows[0]["momentum"])
    g = np.array(sc.parameters.gravity, np.float64)
    out = {"mass_initial": m0, "mass_final": rows[-1]["mass"],
           "mass_drift_rel": (rows[-1]["mass"] - m0) / m0,
           "kinetic_energy_initial": rows[0]["kinetic_energy"], "kinetic_energy_final": rows[-1]["kinetic_energy"]}
    splits = sum(r["splits"] for r in refinements)
    if refinements:
        # mass changes only where particles split (13 x 0.077 = 1.001 of the parent: +0.001 m_parent per split, the
        # reference's mass ratios) and by the rounding of merged masses (m1 + m2 in FP32)
        out["splits"] = splits
        out["merges"] = sum(r["merge_pairs"] for r in refinements)
        out["mass_gain_per_split_over_m0"] = ((rows[-1]["mass"] - m0) / splits / sc.parameters.base_particle_mass
                                              if splits else None)
        out["split_mass_ratio_excess"] = 13 * 0.077 - 1.0
    # momentum minus the impulse of gravity on the whole mass: what walls and the domain clamp added (zero, to
    # rounding, where nothing but pair forces act)
    t_end = rows[-1]["frame"] * sc.dt
    wall = np.array(rows[-1]["momentum"]) - P0 - g * m0 * t_end
    out["momentum_minus_gravity_impulse_final"] = wall.tolist()
    out["momentum_abs_max_over_run"] = float(max(np.abs(np.array(r["momentum"])).max() for r in rows))
    return out


def run_conservation(args, rank: int, world: int, dist):
    """FP64 mass, momentum and kinetic energy over --drift-steps steps (default 10,000) of: the 1M adaptive dam break
    (refinement on: mass changes only at split events, Q-7), the 128k plain dam break (refinement off: the mass is
    constant) and a periodic Taylor-Green vortex at 64^3 (no gravity, no walls: momentum is conserved up to
    rounding). Totals every --drift-every steps from fixed-order FP64 reductions on the device."""
    import torch

    from adaptivesph_gb300 import scenes

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if rank != 0:
        return None
    cases = [("adaptive dam break 1M (100x200x50, dx=0.004 m), velocity criterion", c2_scene(args), True),
             ("plain dam break 128k (40x80x40, dx=0.01 m)", scenes.c1_plain(), False),
             ("periodic Taylor-Green vortex 64^3, Re=100, Morris viscosity", scenes.taylor_green(64), False)]
    results = []
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    for name, sc, adaptive in cases:
        rows, refs, secs, errors = _conservation_run(sc, args.drift_steps, args.drift_every, adaptive)
        results.append({"case": name, "steps": args.drift_steps, "dt": sc.dt, "seconds": secs,
                        "device_errors": errors, "summary": _drift_summary(rows, refs, sc, args.drift_every),
                        "totals": rows, "refinements": refs})
    clocks = sampler.stop()
    line = {"metric": "FP64 conserved totals over 10k steps", "workload": "conservation",
            "steps": args.drift_steps, "every": args.drift_every, "n_gpus": 1, "clocks": clocks, "cases": results}
    if args.out:
        with open(args.out, "w") as f:
            json.dump(line, f, indent=1)
    return {k: v for k, v in line.items() if k != "cases"} | {
        "cases": [{"case": r["case"], "seconds": r["seconds"], "summary": r["summary"]} for r in results]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-steps", type=int, default=10, help="steps of the CPU baseline sample in the GPU arm")
    ap.add_argument("--ref-steps", type=int, default=40, help="most steps the reference arm times")
    ap.add_argument("--no-late", action="store_true", help="skip the late-frame leg")
    ap.add_argument("--late-frame", type=int, default=150, help="first frame of the late-frame leg")
    ap.add_argument("--criterion", choices=["velocity", "free_surface"], default="velocity",
                    help="split/merge criterion of the 1M adaptive dam break: the reference's velocity criterion, or "
                         "the neighbour-count deficit that splits at the free surface")
    ap.add_argument("--plain-steps", type=int, default=200,
                    help="frames of the plain-form legs (ours, and the reference's CUDA step in the reference arm)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--drift-steps", type=int, default=10000, help="steps of the conservation workload")
    ap.add_argument("--drift-every", type=int, default=100, help="steps between FP64 totals (conservation)")
    ap.add_argument("--out", default="", help="conservation: write the full record (every totals row) to this file")
    ap.add_argument("--workload", choices=["adaptive1m", "batched", "served", "conservation", "batch1m"],
                    default="adaptive1m",
                    help="adaptive1m: the headline 1M adaptive dam break; batched: the scene mix through asph_batch; "
                         "served: Poisson scene requests through asph_server; batch1m: the 1M plain dam break alone in "
                         "a batch (--batch-mode)")
    ap.add_argument("--batch-mode", choices=["auto", "graphs", "segmented"], default="segmented",
                    help="batch mode of the batch1m workload")
    ap.add_argument("--requests", type=int, default=24, help="requests of the served workload")
    ap.add_argument("--rates", type=float, nargs="+", default=[5.0, 10.0, 20.0, 50.0, 100.0, 200.0],
                    help="arrival rates (1/s)")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="device-memory budget of the server")
    ap.add_argument("--poll-steps", type=int, default=50, help="steps per server poll")
    ap.add_argument("--scenes", type=int, default=256, help="scenes of the batched mix")
    ap.add_argument("--capacity", type=int, default=0,
                    help="particle capacity (default: the workload's 4M); a smaller one keeps profiling runs small")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl")
        dist = tdist
    runners = {"batched": run_batched, "served": run_served, "adaptive1m": run_ours,
               "conservation": run_conservation, "batch1m": run_batch_one}
    line = runners[args.workload](args, rank, world, dist)
    if line is not None:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
