"""Benchmark of the GB300 position-based-fluids step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the 1,048,576-particle single scene): a 128 x 128 x 64 block of
particles at spacing 0.05 (h = 0.1) in a 6.4 m cube with 64^3 cells, the
paper equations (relaxation 600, s_corr k 0.1 n 4 dq 0.2 h, XSPH 0.01,
vorticity 0.0005), 4 solver iterations, dt = 1/120, seeded jitter.  A step
is one full simulation step (hash, sort, cell ranges, reorder, 4 x lambda
and delta-p, vorticity, XSPH + commit).  The metric is particle-iterations/s
= N particles x 4 solver iterations x steps / seconds.

Our arm prints one JSON line with:
  value     device-resident throughput: K steps replayed as CUDA graphs,
            timed with CUDA events on the simulation's stream;
  e2e       the same metric through the C-ABI with host buffers: every step
            uploads the state from page-locked host memory, steps, and reads
            the state back, all inside the timed region; over the first (up
            to 20) of the timed steps, from their start state;
  roofline  the dominant kernel's algorithmic bytes per launch over its
            average launch time (a second timed pass with an event after
            every launch), against the measured HBM copy bandwidth;
  density_error  the density constraint's error in the final state
            (mean and max compression, interior mean |rho/rho0 - 1|), read
            back after the timed region;
  neighbour_lists  the final step's largest neighbour count and how many
            particles exceeded the list capacity (and re-derived their sets);
  fp64_step_error  one step from the timed steps' start state and one from
            their final state against the FP64 oracle of the same equations
            from the same state (largest position difference in h, its
            distribution; the bound is 1e-5 h), beside the same step in
            binary32 on the host, untimed;
  equations "paper": the line's value runs Macklin & Mueller's equations;
  ref_equations  the same scene in REF_COMPAT mode (the reference kernels'
            own equations, bit-exact with them): device-resident and end to
            end through the C-ABI with host buffers, steps 1..20 from the
            initial state -- the like-for-like figure beside the reference
            arm, which can only run the reference's equations;
  cpu_baseline  the reference's own kernels (compiled from their sources)
            or, where they are absent, the oracle's restatement of them, on a
            bounded sample of the same workload on the host cores (the scene
            built by the oracle's own generator: the CPU legs load nothing of
            the product library).
The working set (state, neighbour lists, sort buffers) is several hundred MB,
larger than L2, so no flush runs between steps.

  forms     (default) the batched and served workloads below, summarised:
            value, vs the same scenes solved one by one on the plain path,
            scene latency.
Before warm-up each workload runs the launch-shape tuner on its own scenes
(--no-tune keeps the defaults; results are bitwise the same either way).

--workload small: the 32,768-particle dam break (32^3 block in a 1.6 x 1.6
x 3.2 box), 500 steps; its reference arm runs the paper equations of that
configuration on the host cores for all 500 steps (the oracle's binary32
restatement: the reference's kernels have no s_corr or vorticity) beside
the reference's own kernels for their first 20 steps.

--workload batch: 256 independent dam breaks, N log-uniform 4,096..262,144,
block aspect ratios in [0.5, 2], boxes twice the block extent, advanced
together for 300 steps (one launch per kernel per step, CUDA graph); against
each scene alone on the plain path.
--workload serve: a seeded Poisson stream (mean 50 requests/s) of dam-break
solves, N log-uniform 8,192..524,288, 100..1000 steps each, submitted in
real time for --serve-seconds to the request loop (continuous batching
under a 120 GB HBM budget); p50/p99 completion latency; against the same
requests solved one at a time on the plain path.
--workload aux: the rows around the step on the 1M scene (scenario file
I/O text vs binary, the headless runner's snapshot cost, a 1280 x 720
render), printed as one line with "metric": "aux".
--save-state / --load-state write and resume the single scene's state (for
profiling a late state of the simulation); --max-neighbours sets the
neighbour-list capacity of the single and large scenes (particles with more
neighbours re-derive their sets in every pass).

--impl reference times the reference's own CPU implementation on the same
workload and prints the same line with "impl": "reference".
Under torchrun (N > 1) every rank runs an independent replica of the scene
(replicas only: a single scene is not sharded); value sums all ranks' work
over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ITERATIONS = 4
METRIC = "particle-iterations/s"
UNIT = "particle-iterations/s"
# Compulsory HBM bytes per particle and launch of each stage (neighbour
# re-reads counted as cache hits): predict+hash 72, sort 4 + 16 per digit
# pass (36 for the 18-bit keys of a 64^3 grid: two 9-bit passes), cell
# ranges 8, reorder 104, lambda 24, delta-p 36, vorticity 48, XSPH+commit 84;
# 556 + the sort per particle-step in total (592 on a 64^3 grid).  The
# neighbour-list build (read p* 16, write the count 4) is an implementation
# choice outside that total; fused with the first lambda it counts both
# (20 + 24).  Every kernel the step launches has an entry, so the roofline
# object names the kernel that takes the most time.
ALG_BYTES = {
    "predict_hash": 72, "sort_onesweep": 36, "cell_offsets": 8, "cell_sort": 22, "reorder": 104,
    "nbr_build": 20, "nbr_lambda": 44, "lambda": 24, "delta": 36, "vorticity": 48,
    "xsph_commit": 84,
}
STEP_BYTES_BUT_SORT = 556  # with the radix sort's cell offsets (8), without the sort


def sort_passes(key_bits: int) -> int:
    """Digit passes of the radix sort: 9-bit digits for 9 and 17-18 key bits
    (where they save a pass within two passes), 8-bit ones otherwise."""
    w = 9 if key_bits in (9, 17, 18) else 8
    return -(-key_bits // w)


def sort_key_bits(cells: int) -> int:
    return max(1, int(np.ceil(np.log2(max(cells, 2)))))


def sort_bytes(cells: int) -> int:
    return 4 + 16 * sort_passes(sort_key_bits(cells))


def cell_sort_bytes(particles: int, cells: int) -> int:
    """The counting sort by cell (the default sort of the step): read the
    keys and each particle's place in its cell (8; the place is written by
    the predict kernel, 4), write the sorted keys and the permutation (8),
    read the counts and write the offsets (8 per cell), rounded."""
    return int(round(20 + 8 * cells / max(particles, 1)))


def step_bytes(cells: int, particles: int = 0, counting: bool = False) -> int:
    if counting:  # the counting sort writes the cell offsets itself
        return STEP_BYTES_BUT_SORT - ALG_BYTES["cell_offsets"] + cell_sort_bytes(particles, cells)
    return STEP_BYTES_BUT_SORT + sort_bytes(cells)


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def density_error_of(sim, rest_density: float, at_step: int) -> dict:
    """The density constraint's error in the state just stepped (from its
    last lambda pass, read back after the timed region): mean and max
    compression max(rho/rho0 - 1, 0), and mean |rho/rho0 - 1| over particles
    away from the free surface (rho >= 0.8 rho0)."""
    rho = sim.density() / rest_density
    comp = np.maximum(rho - 1.0, 0.0)
    interior = rho >= 0.8
    return {"at_step": at_step, "mean_compression": float(comp.mean()),
            "max_compression": float(comp.max()),
            "mean_abs_interior": float(np.abs(rho[interior] - 1.0).mean()) if interior.any() else 0.0}


def profile_traffic(kernel: str):
    """dram read+write bytes per launch and particles per launch of `kernel`
    from the committed ncu summaries (profiles/*.md or *.txt lines of the form
    `traffic kernel=<name> bytes_per_launch=<B> particles=<N>`), or None."""
    for f in sorted([*(ROOT / "profiles").glob("*.txt"), *(ROOT / "profiles").glob("*.md")]):
        for line in f.read_text().splitlines():
            if line.startswith("traffic ") and f"kernel={kernel} " in line + " ":
                kv = dict(t.split("=", 1) for t in line.split()[1:] if "=" in t)
                return float(kv["bytes_per_launch"]), float(kv["particles"])
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu_index = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


# ------------------------------------------------------------------ helpers
def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def make_group(world: int, backend: str):
    if world <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def reduce_max(dist, value: float, device=None) -> float:
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class EventTimer:
    """Device time on one CUDA stream (events recorded on it)."""

    def __init__(self, stream):
        import torch

        self.stream = stream
        self.e0 = torch.cuda.Event(enable_timing=True)
        self.e1 = torch.cuda.Event(enable_timing=True)

    def start(self):
        self.e0.record(self.stream)

    def stop(self) -> float:
        self.e1.record(self.stream)
        self.e1.synchronize()
        return self.e0.elapsed_time(self.e1) / 1e3


class WallTimer:
    """Host wall time (for replicas whose step is not a CUDA stream)."""

    def start(self):
        self.t0 = time.perf_counter()

    def stop(self) -> float:
        return time.perf_counter() - self.t0


def timed_replica_steps(dist, sim, steps: int, timer, particles: int, device=None,
                        before=None) -> tuple[float, float]:
    """Times `steps` steps of this rank's replica: a barrier over the ranks,
    everything before it finished (`before`, e.g. torch.cuda.synchronize),
    the steps enqueued between the timer's marks, then the slowest rank's
    time.  Returns (seconds, value) with value = the particle-iterations of
    every rank's replica over that time (replicas are independent: weak
    scaling)."""
    world = dist.get_world_size() if dist is not None else 1
    if dist is not None:
        dist.barrier()
    if before is not None:
        before()
    sim.sync()
    timer.start()
    sim.step(steps, sync=False)
    t = timer.stop()
    sim.sync()
    t = reduce_max(dist, t, device=device)
    return t, world * particles * ITERATIONS * steps / t


def cpu_reference_run(n_steps_max: int = 50, budget_s: float = 15.0, threads: int = 0,
                      workload: str = "single"):
    """Times the reference's own kernels (or the oracle restatement where
    they are not built) on the workload's scene, one step at a time until
    `budget_s` of CPU time is spent.  The scene comes from the oracle's own
    generator (bit-identical to the library's, checked by the CPU tests), so
    this leg loads nothing of the product library.  Returns (value, info)."""
    import oracle

    cfg, pos, vel = {"large": oracle.scene_4m, "small": oracle.scene_small}.get(
        workload, oracle.scene_1m)()
    n = pos.shape[0]
    threads = threads or (os.cpu_count() or 1)
    kind = "reference" if oracle.reference_available() else "port"
    steps = 0
    t0 = time.perf_counter()
    while steps < n_steps_max:
        if kind == "reference":
            pos, vel, *_ = oracle.reference_steps(cfg, pos, vel, 1, threads=threads, parallel_cells=True)
        else:
            pos, vel, _, _ = oracle.refcompat_steps_f32(cfg, pos, vel, 1, threads=threads)
        steps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    value = n * ITERATIONS * steps / dt
    info = {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "equations": "reference",
            "steps": steps,
            "sample": f"{steps} step(s) of the {n}-particle scene from its initial state, "
                      f"reference equations, {'reference kernels compiled from their .cl sources' if kind == 'reference' else 'oracle restatement of the reference kernels'}, "
                      f"{dt:.1f} s"}
    return value, info


def cpu_paper_run(steps: int, threads: int = 0, workload: str = "small", chunk: int = 25):
    """The paper equations of the benchmark configuration on the host cores:
    the oracle's binary32 restatement (the reference's kernels have no
    s_corr or vorticity), `steps` steps from the scene's initial state in
    chunks of `chunk`.  Returns (value, info)."""
    import oracle

    cfg, pos, vel = {"large": oracle.scene_4m, "single": oracle.scene_1m}.get(
        workload, oracle.scene_small)()
    prm = oracle.benchmark_paper_params(cfg)
    n = pos.shape[0]
    threads = threads or (os.cpu_count() or 1)
    done = 0
    t0 = time.perf_counter()
    while done < steps:
        k = min(chunk, steps - done)
        pos, vel, *_ = oracle.paper_steps_f64(prm, pos, vel, k, threads=threads, precision="f32")
        done += k
    dt = time.perf_counter() - t0
    value = n * ITERATIONS * done / dt
    finite = bool(np.isfinite(pos).all())
    info = {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "equations": "paper",
            "steps": done, "finite": finite,
            "sample": f"all {done} steps of the {n}-particle scene from its initial state, paper "
                      f"equations, the oracle's binary32 restatement on {threads} threads, {dt:.1f} s"}
    return value, info


# -------------------------------------------------------------------- arms
def run_reference(args) -> int:
    world, rank, _ = dist_info()
    if rank != 0:
        return 0
    if args.workload == "small":
        return run_reference_small(args)
    value, info = cpu_reference_run(n_steps_max=max(1, args.steps), budget_s=args.cpu_budget,
                                    workload=args.workload)
    large = args.workload == "large"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "equations": "reference",
        "config": {"workload": "double_dam_break_4m" if large else "single_scene_1m",
                   "particles": 4194304 if large else 1048576, "cells": 1048576 if large else 262144,
                   "solver_iterations": ITERATIONS,
                   "equations": "reference kernels (relaxation 1e4, no s_corr, XSPH, no vorticity)",
                   "note": "the like-for-like GPU figure is the headline line's ref_equations"},
        "cpu_baseline": info,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_reference_small(args) -> int:
    """The 32,768-particle configuration on the host cores: all its steps in
    the paper equations it names (the oracle's binary32 restatement), and
    the reference's own kernels on the same scene for their first 20 steps
    (its equations push this block out of its box after ~30 steps)."""
    value, info = cpu_paper_run(max(1, args.steps), workload="small")
    _, kernels = cpu_reference_run(n_steps_max=20, budget_s=args.cpu_budget, workload="small")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": info["steps"], "warmup": 0, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "equations": "paper",
        "config": {"workload": "dam_break_32k", "particles": 32768, "cells": 16 * 16 * 32,
                   "box": [1.6, 1.6, 3.2], "solver_iterations": ITERATIONS,
                   "equations": "paper (relaxation 600, s_corr, XSPH, vorticity)"},
        "cpu_baseline": info,
        "reference_kernels": kernels,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def ref_equations_run(pbf, sc, args) -> dict:
    """The same scene through the GPU path in REF_COMPAT mode (the
    reference's own equations, bit-exact with its kernels): the like-for-like
    figure beside the reference arm, which runs those equations on the CPU.
    Both legs time steps 1..20 from the scene's initial state, the sample the
    CPU arm times: device-resident (CUDA graph steps, CUDA events), and end to
    end through the C-ABI with page-locked host buffers (every step uploads
    the state, steps and reads the state back inside the timed region)."""
    import ctypes as C

    import torch

    p = sc.params.copy()
    p.mode = pbf.MODE_REF_COMPAT
    steps = 20
    pos0, vel0 = pbf.state_from_particles(sc.particles)
    n = sc.n
    with pbf.Simulation(p, sc.particles) as sim:
        sim.init()
        sim.initCells()
        sim.step(2)  # module load, graph instantiation
        sim.set_state(pos0, vel0)
        ext = torch.cuda.ExternalStream(sim.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        sim.step(steps, sync=False)
        e1.record(ext)
        e1.synchronize()
        sim.sync()
        t = e0.elapsed_time(e1) / 1e3
        dev_pos, _ = sim.dumpData()
        finite = bool(np.isfinite(dev_pos).all())
        launches = sim.launches_per_step()
        # end to end with host buffers
        hp = pbf.lib()
        nbytes = n * 16
        pin_pos, pin_vel = C.c_void_p(), C.c_void_p()
        hp.pbf_host_alloc(nbytes, C.byref(pin_pos))
        hp.pbf_host_alloc(nbytes, C.byref(pin_vel))
        host_pos = np.frombuffer((C.c_float * (4 * n)).from_address(pin_pos.value), np.float32).reshape(n, 4)
        host_vel = np.frombuffer((C.c_float * (4 * n)).from_address(pin_vel.value), np.float32).reshape(n, 4)
        host_pos[:] = pos0
        host_vel[:] = vel0
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(ext)
        for _ in range(steps):
            sim.set_state_async(pin_pos.value, pin_vel.value)
            sim.step(1, sync=False)
            sim.dump_data_async(pin_pos.value, pin_vel.value)
        f1.record(ext)
        f1.synchronize()
        sim.sync()
        t_e2e = f0.elapsed_time(f1) / 1e3
        same = bool(np.array_equal(host_pos.view(np.uint32), dev_pos.view(np.uint32)))
        del host_pos, host_vel
        hp.pbf_host_free(pin_pos)
        hp.pbf_host_free(pin_vel)
    return {"value": n * ITERATIONS * steps / t, "unit": UNIT, "ms_per_step": t / steps * 1e3,
            "steps": steps, "start_state": "initial block", "gpu_launches": launches * steps,
            "finite": finite, "equations": "reference",
            "e2e": {"value": n * ITERATIONS * steps / t_e2e, "unit": UNIT,
                    "ms_per_step": t_e2e / steps * 1e3, "h2d_bytes_per_step": 2 * nbytes,
                    "d2h_bytes_per_step": 2 * nbytes, "same_result_as_device_resident": same},
            "method": "REF_COMPAT (the reference kernels' equations, bit-exact with them), CUDA-graph "
                      "steps 1..20 from the initial state; e2e through the C-ABI with page-locked "
                      "host buffers, the state up and down every step"}


def fp64_step_error(pbf, sim, params, state=None, where: str = "the state after the timed steps") -> dict:
    """One step of the simulation from `state` (default: its current state)
    against the FP64 oracle of the same equations from the same state
    (outside every timed region): largest position and velocity difference,
    in h and m/s, and how the position differences are distributed."""
    import oracle
    import __graft_entry__ as ge

    pos, vel = state if state is not None else sim.dumpData()
    sim.set_state(pos, vel)
    sim.step(1)
    gpos, gvel = sim.dumpData()
    t0 = time.perf_counter()
    prm = ge.paper_params_for_oracle(params)
    opos, ovel, *_ = oracle.paper_steps_f64(prm, pos, vel, 1)
    ex = np.abs(gpos[:, :3].astype(np.float64) - opos[:, :3]).max(axis=1) / params.h
    dv = np.abs(gvel[:, :3].astype(np.float64) - ovel[:, :3]).max()
    # the same step evaluated in binary32 on the host (IEEE operations, the
    # oracle's own order): how far binary32 itself lands from FP64 here
    cpos, *_ = oracle.paper_steps_f64(prm, pos, vel, 1, precision="f32")
    cx = np.abs(cpos[:, :3] - opos[:, :3]).max(axis=1) / params.h
    # particles stacked on one point (clamped into a corner of the box) do
    # not interact (r = 0) and can carry speeds where one step is chaotic
    stacked = int(pos.shape[0] - np.unique(pos[:, :3], axis=0).shape[0])
    return {"position_max_h": float(ex.max()), "position_p999_h": float(np.percentile(ex, 99.9)),
            "particles_over_bound": int((ex > 1e-5).sum()), "velocity_max": float(dv),
            "bound_position_h": 1e-5, "within_bound": bool(ex.max() <= 1e-5),
            "host_binary32": {"position_max_h": float(cx.max()),
                              "position_p999_h": float(np.percentile(cx, 99.9)),
                              "particles_over_bound": int((cx > 1e-5).sum())},
            "stacked_particles": stacked, "oracle_s": time.perf_counter() - t0,
            "method": f"one step from {where}, GPU (binary32) against the FP64 oracle "
                      "restatement of the same equations from the same state"}


def run_ours(args) -> int:
    import torch

    import __graft_entry__ as ge

    world, rank, local = dist_info()
    torch.cuda.set_device(local)
    dist = make_group(world, "nccl")
    pbf = ge.load_package()
    sc = {"large": pbf.scenes.config_4m, "small": pbf.scenes.config_small}.get(
        args.workload, pbf.scenes.config_1m)()
    if args.max_neighbours:
        sc.params.max_neighbours = args.max_neighbours
    n = sc.n
    sim = pbf.Simulation(sc.params, sc.particles)
    sim.init()
    sim.initCells()
    if args.load_state:
        sim.load_state(args.load_state)
    tuning = None if args.no_tune else sim.autotune(3).as_dict()
    if (args.first_pass != "auto" or args.staged != "auto" or args.sort != "auto"
            or args.build != "auto"):
        t = sim.tuning()
        if args.first_pass != "auto":
            t.fuse_first = 1 if args.first_pass == "fused" else 0
        if args.build != "auto":
            t.masked_build = 1 if args.build == "masked" else 0
        if args.staged != "auto":
            t.staged = 1 if args.staged == "on" else 0
        if args.sort != "auto":
            t.radix_sort = 1 if args.sort == "radix" else 0
        sim.set_tuning(t)
        tuning = sim.tuning().as_dict()
    ext = torch.cuda.ExternalStream(sim.stream())
    launches = sim.launches_per_step()

    # warm-up (also instantiates the step graph)
    sim.step(args.warmup)
    # the state the timed steps start from: the per-kernel timing pass below
    # replays the same steps from it
    start_state = sim.dumpData()

    # ---- device-resident throughput ------------------------------------
    with ClockSampler(local) as clocks:
        t_dev, value = timed_replica_steps(dist, sim, args.steps, EventTimer(ext), n, device="cuda",
                                           before=torch.cuda.synchronize)
    clock_summary = clocks.summary()
    if args.save_state and rank == 0:
        sim.save_state(args.save_state)
    density_error = density_error_of(sim, sc.params.rest_density, args.warmup + args.steps)
    nbr_max, nbr_over = sim.neighbour_stats()
    tiles = sim.tile_stats()
    fp64_end = fp64_step_error(pbf, sim, sc.params) if rank == 0 and not args.no_fp64 else None

    # ---- end to end through the C-ABI with host buffers ------------------
    nbytes = n * 16
    hp = pbf.lib()
    import ctypes as C

    pin_pos, pin_vel = C.c_void_p(), C.c_void_p()
    hp.pbf_host_alloc(nbytes, C.byref(pin_pos))
    hp.pbf_host_alloc(nbytes, C.byref(pin_vel))
    # the same steps the device-resident figure starts with: from the timed
    # steps' start state, held in page-locked host memory by the caller
    for ptr, arr in ((pin_pos, start_state[0]), (pin_vel, start_state[1])):
        np.frombuffer((C.c_float * (4 * n)).from_address(ptr.value), np.float32).reshape(n, 4)[:] = arr
    e2e_steps = max(3, min(args.steps, 20))
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(ext)
    for _ in range(e2e_steps):
        sim.set_state_async(pin_pos.value, pin_vel.value)
        sim.step(1, sync=False)
        sim.dump_data_async(pin_pos.value, pin_vel.value)
    f1.record(ext)
    f1.synchronize()
    sim.sync()
    t_e2e = reduce_max(dist, f0.elapsed_time(f1) / 1e3, device="cuda")
    e2e_value = world * n * ITERATIONS * e2e_steps / t_e2e
    final = np.frombuffer((C.c_float * (4 * n)).from_address(pin_pos.value), np.float32).reshape(n, 4)
    finite = bool(np.isfinite(final).all())
    hp.pbf_host_free(pin_pos)
    hp.pbf_host_free(pin_vel)

    # ---- per-kernel timing pass: the timed steps again, from the same ----
    # state, with an event after every launch (each step one graph)
    sim.set_state(*start_state)
    sim.set_stage_timing(True)
    kt_steps = args.steps
    sim.step(kt_steps)
    kt = sim.kernel_times()
    stages = sim.stage_times()
    sim.set_stage_timing(False)
    fp64_err = None
    if fp64_end is not None:
        fp64_err = {"at_start": fp64_step_error(pbf, sim, sc.params, start_state,
                                                f"the timed steps' start state (step {args.warmup})"),
                    "at_end": fp64_end}
    total_ms = sum(ms for ms, _ in kt.values())
    dom = max((k for k in kt if k in ALG_BYTES), key=lambda k: kt[k][0])
    dom_ms, dom_launches = kt[dom]
    per_launch_s = dom_ms / 1e3 / dom_launches
    if dom == "sort_onesweep":
        per_launch_s = dom_ms / 1e3 / kt_steps
    peaks = measured_peaks()
    alg = dict(ALG_BYTES, sort_onesweep=sort_bytes(sc.params.ncells),
               cell_sort=cell_sort_bytes(n, sc.params.ncells))
    counting = "cell_sort" in kt
    achieved = alg[dom] * n / per_launch_s / 1e9
    traffic = profile_traffic(dom)
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
        "traffic": (traffic[0] * n / traffic[1]) if traffic else None,
        "algorithmic_bytes_per_launch": alg[dom] * n,
        "avg_launch_ms": per_launch_s * 1e3, "share_of_step": dom_ms / total_ms,
    }
    step_s = t_dev / args.steps
    sb = step_bytes(sc.params.ncells, n, counting)
    step_roofline = {"bytes_per_particle_step": sb,
                     "achieved_gbs": sb * n / step_s / 1e9,
                     "frac": sb * n / step_s / 1e9 / peaks["hbm_gbs"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        if args.workload == "small":
            _, cpu = cpu_paper_run(min(args.steps, 500), workload="small")
        else:
            _, cpu = cpu_reference_run(budget_s=args.cpu_budget, workload=args.workload)

    sim.close()
    ref_eq = ref_equations_run(pbf, sc, args) if world == 1 else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "equations": "paper",
            "config": {"workload": sc.name, "particles": n, "cells": sc.params.ncells,
                       "box": sc.meta["box"], "blocks": sc.meta.get("blocks", [sc.meta.get("block")]),
                       "solver_iterations": ITERATIONS,
                       "equations": "paper (relaxation 600, s_corr, XSPH, vorticity)",
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "working set larger than L2; no flush between steps",
                       "graph": True, "start_state": args.load_state or "initial block",
                       "list_capacity": int(sc.params.max_neighbours),
                       "tuning": tuning},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes,
                    "d2h_bytes_per_step": 2 * nbytes, "steps": e2e_steps,
                    "start_state": f"the timed steps' start state (step {args.warmup})",
                    "finite": finite},
            "gpu_launches": launches * args.steps,
            "roofline": roofline,
            "step_roofline": step_roofline,
            "stage_ms": {"sort": float(stages[0]), "lambda": float(stages[1]), "delta_p": float(stages[2]),
                         "velocity": float(stages[3])},
            "kernel_ms_per_step": {k: v[0] / kt_steps for k, v in kt.items()},
            "kernel_timing": {"steps": kt_steps, "sum_ms_per_step": total_ms / kt_steps,
                              "method": "the timed steps replayed from their start state, each "
                                        "step one graph with an event after every launch"},
            "clocks": clock_summary,
            "density_error": density_error,
            "fp64_step_error": fp64_err,
            "neighbour_lists": {"capacity": int(sc.params.max_neighbours), "max_count": nbr_max,
                                "overflow": nbr_over, "at_step": args.warmup + args.steps},
            "staged_tiles": {"staged": tiles[0], "unstaged": tiles[1], "at_step": args.warmup + args.steps},
            "cpu_baseline": cpu,
            "ref_equations": ref_eq,
        }
        if args.forms == "all" and world == 1 and args.workload == "single":
            line["forms"] = form_summaries(args)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def with_sort(obj, sort: str):
    """Sets the step's cell sort of a simulation or batch ("counting" or
    "radix"; "auto" keeps the library's default, the counting sort)."""
    if sort != "auto":
        t = obj.tuning()
        t.radix_sort = 1 if sort == "radix" else 0
        obj.set_tuning(t)
    return obj


def plain_one_by_one(pbf, scenes, steps, sample_steps: int, ext_stream_of, sort: str = "auto"):
    """The scenes solved one at a time on the plain path: per scene, create,
    upload, warm up (3 steps), then time its steps as graph-replayed steps
    with CUDA events -- all of them (`sample_steps` 0), or the first
    `sample_steps` scaled to the scene's count.  `steps` is one count for
    every scene or one per scene.  Returns per-scene seconds for its steps and
    the wall seconds of set-up plus read-back per scene."""
    import torch

    step_s, setup_s = [], []
    for i, s in enumerate(scenes):
        n_steps = steps[i] if isinstance(steps, (list, tuple)) else steps
        timed = n_steps if sample_steps <= 0 else max(1, min(sample_steps, n_steps))
        w0 = time.perf_counter()
        sim = pbf.Simulation(s.params, s.particles)
        sim.init()
        with_sort(sim, sort)
        sim.step(3)
        ext = ext_stream_of(sim)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        sim.step(timed, sync=False)
        e1.record(ext)
        e1.synchronize()
        sim.sync()
        t = e0.elapsed_time(e1) / 1e3 / timed * n_steps
        sim.dumpData()
        sim.close()
        step_s.append(t)
        setup_s.append(time.perf_counter() - w0 - e0.elapsed_time(e1) / 1e3)
    return step_s, setup_s


def plain_by_size(sizes, plain_step_s, steps: int, t_batch: float) -> list:
    """The plain one-by-one time by scene size: per bucket of particle
    counts, the scenes, their share of the particles, their share of the
    plain time, their plain rate and the ratio the batch would show on them
    alone at its whole-mix rate per particle."""
    sizes = np.asarray(sizes)
    secs = np.asarray(plain_step_s)
    total_n, total_t = sizes.sum(), secs.sum()
    out = []
    for lo, hi in ((0, 32768), (32768, 131072), (131072, 1 << 31)):
        sel = (sizes >= lo) & (sizes < hi)
        if not sel.any():
            continue
        n, t = int(sizes[sel].sum()), float(secs[sel].sum())
        rate = n * ITERATIONS * steps / t
        out.append({"particles": [lo, min(hi, int(sizes.max()))], "scenes": int(sel.sum()),
                    "particle_share": float(n / total_n), "plain_time_share": float(t / total_t),
                    "plain_value": float(rate),
                    "batch_over_plain": float((total_n * ITERATIONS * steps / t_batch) / rate)})
    return out


def run_batch(args, emit: bool = True):
    """256 independent dam-break scenes of log-uniform sizes advanced together
    (one launch per kernel per step, CUDA-graph step) against the same scenes
    solved one at a time on the plain path."""
    import torch

    import __graft_entry__ as ge

    world, rank, local = dist_info()
    torch.cuda.set_device(local)
    dist = make_group(world, "nccl")
    pbf = ge.load_package()
    scenes = pbf.scenes.mixed_batch(256)
    steps = args.steps
    n_tot = sum(s.n for s in scenes)
    cells_tot = sum(s.params.ncells for s in scenes)
    solver = scenes[0].params

    # ---- end to end: upload every scene, step, read every scene back ------
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    b = pbf.Batch(solver, len(scenes), n_tot, cells_tot)
    ids = [b.add_scene(s.params, s.particles) for s in scenes]
    tuning = None if args.no_tune else b.autotune(3).as_dict()
    if args.sort != "auto":
        tuning = with_sort(b, args.sort).tuning().as_dict()
    ext = torch.cuda.ExternalStream(b.stream())
    launches = b.launches_per_step()
    b.step(args.warmup)
    b.sync()
    # ---- device-resident throughput ------------------------------------
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        e0.record(ext)
        b.step(steps, sync=False)
        e1.record(ext)
        e1.synchronize()
    b.sync()
    finite = all(bool(np.isfinite(b.dump_scene(i)[0]).all()) for i in ids)
    t_wall = time.perf_counter() - w0
    b.close()
    t_dev = reduce_max(dist, e0.elapsed_time(e1) / 1e3, device="cuda")
    value = world * n_tot * ITERATIONS * steps / t_dev
    work_e2e = n_tot * ITERATIONS * (steps + args.warmup)
    t_wall = reduce_max(dist, t_wall, device="cuda")
    e2e_value = world * work_e2e / t_wall
    peaks = measured_peaks()
    batch_step_bytes = step_bytes(cells_tot, n_tot, counting=not (tuning or {}).get("radix_sort", 0))
    step_gbs = batch_step_bytes * n_tot / (t_dev / steps) / 1e9

    # ---- the same scenes one by one on the plain path ---------------------
    plain = None
    if rank == 0 and not args.no_plain:
        sample = args.plain_sample
        plain_step_s, plain_setup_s = plain_one_by_one(
            pbf, scenes, steps, sample, lambda sim: torch.cuda.ExternalStream(sim.stream()),
            args.sort)
        t_plain = sum(plain_step_s)
        done = np.cumsum([a + c for a, c in zip(plain_step_s, plain_setup_s)])
        plain = {"value": n_tot * ITERATIONS * steps / t_plain, "unit": UNIT,
                 "seconds_device": t_plain,
                 "scene_latency_s": {"p50": float(np.percentile(done, 50)),
                                     "p99": float(np.percentile(done, 99))},
                 "by_scene_size": plain_by_size([s.n for s in scenes], plain_step_s, steps, t_dev),
                 "method": f"each scene alone through the plain C-ABI path (CUDA-graph steps); "
                           + (f"all {steps} steps of each scene timed after 3 warm-up steps; " if sample <= 0
                              else f"{sample} timed steps per scene after 3 warm-up steps, scaled to {steps}; ")
                           + f"latency = completion time of scene k when solved in sequence"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": args.warmup, "ms_per_step": t_dev / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch_256_scenes", "scenes": len(scenes), "particles": n_tot,
                       "cells": cells_tot, "sizes": "log-uniform 4096..262144, seed 0x5EED",
                       "solver_iterations": ITERATIONS, "graph": True, "tuning": tuning,
                       "equations": "paper (relaxation 600, s_corr, XSPH, vorticity)",
                       "l2": "working set larger than L2; no flush between steps"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 32 * n_tot / (steps + args.warmup),
                    "d2h_bytes_per_step": 32 * n_tot / (steps + args.warmup),
                    "method": "wall clock from batch creation through upload of every scene, "
                              f"{args.warmup}+{steps} steps and read-back of every scene",
                    "finite": finite},
            "gpu_launches": launches * steps,
            "step_roofline": {"bytes_per_particle_step": batch_step_bytes, "achieved_gbs": step_gbs,
                              "frac": step_gbs / peaks["hbm_gbs"], "peak_source": peaks["source"]},
            "scene_latency_s": {"p50": t_wall, "p99": t_wall,
                                "note": "every scene of the batch completes with the last step"},
            "plain_one_by_one": plain,
            "speedup_vs_plain": (value / plain["value"]) if plain else None,
            "clocks": clocks.summary(),
        }
        if emit:
            print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return line if not emit else 0


def fifo_latencies(arrivals, service):
    """Completion latency of each job on one server taking jobs in arrival
    order, given arrival times and service times (seconds)."""
    t = 0.0
    lat = []
    for a, s in zip(arrivals, service):
        t = max(t, a) + s
        lat.append(t - a)
    return lat, t


def run_serve(args, emit: bool = True):
    """A seeded Poisson stream of dam-break solves (mean 50 per second, N
    log-uniform 8,192..524,288, 100..1000 steps) submitted in real time to
    the request loop (continuous batching under a 120 GB HBM budget), against
    the same requests solved one by one on the plain path."""
    import torch

    import __graft_entry__ as ge

    world, rank, local = dist_info()
    torch.cuda.set_device(local)
    pbf = ge.load_package()
    rate = getattr(args, "serve_rate", 50.0)
    reqs = pbf.scenes.request_stream(args.serve_seconds, rate=rate)
    work = {r.index: r.n * r.steps * ITERATIONS for r in reqs}
    solver = reqs[0].scene().params
    budget = int(args.hbm_budget_gb * 1e9)
    srv = pbf.Server(solver, budget, max_scenes=4096, cells_per_particle=2.0, max_chunk=args.max_chunk)
    cap = srv.stats()
    # warm the kernels once (module load, graph instantiation) before the clock starts
    w = pbf.scenes.block_in_double_box((8, 8, 8), 1, 3, "warm")
    srv.submit(w.params, w.particles, 3)
    for rid in srv.run_until_idle():
        srv.result(rid)

    submitted = {}
    done_at = {}
    scenes = {}
    i = 0
    t0 = time.perf_counter()
    with ClockSampler(local) as clocks:
        busy = True
        while i < len(reqs) or busy:
            now = time.perf_counter() - t0
            while i < len(reqs) and reqs[i].arrival <= now:
                sc = reqs[i].scene()
                rid = srv.submit(sc.params, sc.particles, reqs[i].steps)
                submitted[rid] = reqs[i]
                i += 1
            ids, busy = srv.poll(wait=False)
            t_now = time.perf_counter() - t0
            for rid in ids:
                done_at[rid] = t_now
                pos, _ = srv.result(rid)
                scenes[rid] = bool(np.isfinite(pos).all())
            if not ids:
                time.sleep(0.0005)
    st = srv.stats()
    srv.close()
    lat = [done_at[rid] - r.arrival for rid, r in submitted.items()]
    makespan = max(done_at.values()) - reqs[0].arrival
    total_work = sum(work.values())
    value = total_work / makespan

    plain = None
    if not args.no_plain:
        sample = args.plain_sample
        plain_step_s, plain_setup_s = plain_one_by_one(
            pbf, [r.scene() for r in reqs], [r.steps for r in reqs], sample,
            lambda sim: torch.cuda.ExternalStream(sim.stream()))
        service = [ps + su for ps, su in zip(plain_step_s, plain_setup_s)]
        plat, pend = fifo_latencies([r.arrival for r in reqs], service)
        plain = {"value": total_work / (pend - reqs[0].arrival), "unit": UNIT,
                 "scene_latency_s": {"p50": float(np.percentile(plat, 50)),
                                     "p99": float(np.percentile(plat, 99))},
                 "method": f"each request alone through the plain C-ABI path: measured set-up and read-back, "
                           f"{'all its' if sample <= 0 else sample} CUDA-event-timed graph steps after 3 "
                           f"warm-up steps{'' if sample <= 0 else ' scaled to its step count'}; latencies "
                           f"from these service times in arrival order (one at a time)"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": int(st["batch_steps"]),
        "warmup": 1, "ms_per_step": makespan / max(1, st["batch_steps"]) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "served_poisson", "rate_per_s": rate, "arrival_window_s": args.serve_seconds,
                   "requests": len(reqs), "n": "log-uniform 8192..524288", "steps": "uniform 100..1000",
                   "hbm_budget_bytes": budget, "batch_capacity_particles": cap["max_particles"],
                   "batch_device_bytes": cap["device_bytes"], "max_chunk": args.max_chunk,
                   "note": "arrivals for the stated window, then the loop drains; throughput = all "
                           "requests' particle-iterations / (last completion - first arrival)"},
        "e2e": {"value": value, "unit": UNIT,
                "h2d_bytes_per_step": 32 * sum(r.n for r in reqs) / max(1, st["batch_steps"]),
                "d2h_bytes_per_step": 32 * sum(r.n for r in reqs) / max(1, st["batch_steps"]),
                "method": "wall clock; particles uploaded at admission, results read back at completion",
                "finite": all(scenes.values())},
        "scene_latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                            "max": float(max(lat))},
        "gpu_launches": int(st["launches"]),
        "server": {k: int(v) for k, v in st.items()},
        "plain_one_by_one": plain,
        "speedup_vs_plain": (value / plain["value"]) if plain else None,
        "clocks": clocks.summary(),
    }
    if not emit:
        return line
    print(json.dumps(line), flush=True)
    return 0


def form_summaries(args) -> dict:
    """The batched and served workloads, summarised for the headline line."""
    import copy

    out = {}
    a = copy.copy(args)
    a.steps = 300
    b = run_batch(a, emit=False)
    if b:
        out["batched"] = {
            "workload": b["config"]["workload"], "scenes": b["config"]["scenes"],
            "particles": b["config"]["particles"], "steps": b["steps"], "value": b["value"],
            "unit": b["unit"], "ms_per_step": b["ms_per_step"], "e2e": b["e2e"]["value"],
            "plain_one_by_one": b["plain_one_by_one"]["value"] if b["plain_one_by_one"] else None,
            "plain_by_scene_size": (b["plain_one_by_one"]["by_scene_size"]
                                    if b["plain_one_by_one"] else None),
            "speedup_vs_plain": b["speedup_vs_plain"], "scene_latency_s": b["scene_latency_s"]["p50"],
            "gpu_launches": b["gpu_launches"], "clocks": b["clocks"]}
    def served_summary(s):
        return {
            "workload": s["config"]["workload"], "rate_per_s": s["config"]["rate_per_s"],
            "requests": s["config"]["requests"],
            "arrival_window_s": s["config"]["arrival_window_s"], "value": s["value"], "unit": s["unit"],
            "scene_latency_s": s["scene_latency_s"],
            "plain_one_by_one": ({"value": s["plain_one_by_one"]["value"],
                                  "scene_latency_s": s["plain_one_by_one"]["scene_latency_s"]}
                                 if s["plain_one_by_one"] else None),
            "speedup_vs_plain": s["speedup_vs_plain"], "hbm_budget_bytes": s["config"]["hbm_budget_bytes"],
            "gpu_launches": s["gpu_launches"], "clocks": s["clocks"]}

    # the benchmark's stream (mean 50 requests/s), which offers about three
    # times what one GB300 serves: throughput, latencies dominated by queueing
    s = run_serve(copy.copy(args), emit=False)
    out["served"] = served_summary(s)
    # the same kind of stream at 0.8 of the rate the first run sustained, so
    # that p50/p99 measure service (batched with the other active requests),
    # not a growing queue
    a = copy.copy(args)
    import __graft_entry__ as ge

    reqs = ge.load_package().scenes.request_stream(args.serve_seconds)
    mean_work = float(np.mean([r.n * r.steps * ITERATIONS for r in reqs]))
    a.serve_rate = round(0.8 * s["value"] / mean_work, 2)
    a.serve_seconds = args.steady_seconds
    out["served_steady"] = served_summary(run_serve(a, emit=False))
    out["served_steady"]["offered_load_vs_capacity"] = 0.8
    return out


def run_aux(args) -> int:
    """The rows around the step, on the 1M-particle scene: scenario files
    (write and read, text .in and binary; host), the headless runner's
    per-step time with no snapshots, binary VTK snapshots and text .in
    snapshots every 10 steps (pbf_run, 120 steps, the snapshots copied into
    page-locked buffers and written by host threads while stepping goes
    on), and one 1280 x 720 point-sprite frame (device time plus read-back;
    median of 7)."""
    import re

    import torch

    import __graft_entry__ as ge

    world, rank, local = dist_info()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    pbf = ge.load_package()
    sc = pbf.scenes.config_1m()
    out = {"metric": "aux", "workload": "aux_1m", "particles": sc.n}
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        io = {}
        for kind, binary in (("text", False), ("binary", True)):
            f = d / f"scene_{kind}.in"
            t0 = time.perf_counter()
            pbf.write_particles(f, sc.particles, binary=binary)
            t1 = time.perf_counter()
            back = pbf.read_particles(f)
            t2 = time.perf_counter()
            assert np.array_equal(back["x"], sc.particles["x"])
            io[kind] = {"write_s": t1 - t0, "read_s": t2 - t1, "bytes": f.stat().st_size}
        out["scenario_io"] = io
        runner = {}
        for label, part_freq, vtk_freq in (("no snapshots", 0, 0), ("vtk every 10 steps", 0, 10),
                                           (".in every 10 steps", 10, 0)):
            p = sc.params.copy()
            p.part_input_file = b"scene_binary.in"
            p.time_end = np.float32(120.5 * p.time_step_length)
            p.part_out_freq = part_freq
            p.part_out_name_base = str(d / "snap_").encode()
            p.vtk_out_freq = vtk_freq
            p.vtk_out_name_base = str(d / "frame_").encode()
            pbf.write_config(d / "scene.par", p)
            t0 = time.perf_counter()
            r = subprocess.run([str(pbf.PKG_DIR / "pbf_run"), str(d / "scene.par")],
                               capture_output=True, text=True, timeout=600)
            wall = time.perf_counter() - t0
            if r.returncode != 0:
                raise RuntimeError(r.stderr)
            mean = float(re.search(r"mean:\s*([0-9.eE+-]+)", r.stdout).group(1))
            runner[label] = {"mean_step_s": mean, "wall_s": wall,
                             "files": len(list(d.glob("snap_*"))) + len(list(d.glob("frame_*")))}
            for f in [*d.glob("snap_*"), *d.glob("frame_*")]:
                f.unlink()
        base = runner["no snapshots"]["mean_step_s"]
        for v in runner.values():
            v["vs_no_snapshots"] = v["mean_step_s"] / base
        out["runner"] = runner
    with pbf.Simulation(sc.params, sc.particles) as sim:
        sim.init()
        sim.step(10)
        sim.render(width=1280, height=720)
        times = []
        for _ in range(7):
            t0 = time.perf_counter()
            img = sim.render(width=1280, height=720)
            times.append(time.perf_counter() - t0)
    out["render"] = {"width": 1280, "height": 720, "median_ms": statistics.median(times) * 1e3,
                     "lit_fraction": float((img.max(axis=2) > 0).mean())}
    print(json.dumps(out), flush=True)
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 500 for the single scene, 300 for the batch)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["single", "small", "large", "batch", "serve", "aux"],
                    default="single",
                    help="single: the 1M-particle scene (headline); small: the 32,768-particle "
                         "dam break; large: the 4.2M-particle double dam break; batch; serve; "
                         "aux: scenario I/O, runner snapshots and rendering around the 1M step")
    ap.add_argument("--serve-seconds", type=float, default=6.0, help="arrival window of the served stream")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="mean requests per second of the served stream")
    ap.add_argument("--steady-seconds", type=float, default=20.0,
                    help="arrival window of the steady-state served run (0.8 of the capacity the "
                         "benchmark stream showed) in the headline line's forms")
    ap.add_argument("--hbm-budget-gb", type=float, default=120.0, help="HBM budget of the request loop")
    ap.add_argument("--max-chunk", type=int, default=16, help="most batched steps per loop turn")
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU baseline work")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the one-step comparison with the FP64 oracle after the timed steps")
    ap.add_argument("--plain-sample", type=int, default=0,
                    help="timed steps per scene of the one-by-one plain comparison, scaled to the "
                         "scene's step count (0, the default: every step of every scene)")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-by-one plain comparison")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--staged", choices=["auto", "on", "off"], default="auto",
                    help="single and large scenes: gather passes on staged shared-memory tiles, "
                         "through L1, or the tuner's (or default) choice")
    ap.add_argument("--sort", choices=["auto", "counting", "radix"], default="auto",
                    help="the step's cell sort: the counting sort by cell (the default) or the "
                         "onesweep radix sort (same permutation); single, large and batch "
                         "workloads and the plain one-by-one comparison")
    ap.add_argument("--first-pass", choices=["auto", "fused", "split"], default="auto",
                    help="single and large scenes: list build fused with the first lambda pass, "
                         "apart from it, or the tuner's (or default) choice")
    ap.add_argument("--build", choices=["auto", "masked", "scan"], default="auto",
                    help="single and large scenes: the list build testing each row into a "
                         "membership mask before storing members, storing members as they are "
                         "found, or the tuner's (or default) choice (same lists)")
    ap.add_argument("--forms", choices=["all", "none"], default="all",
                    help="single workload: also run the batched and served workloads and "
                         "summarise them in the line (one GPU only)")
    ap.add_argument("--save-state", default=None,
                    help="single scene: write the state after the warm-up and timed steps (.npz)")
    ap.add_argument("--load-state", default=None,
                    help="single scene: start from a state written by --save-state")
    ap.add_argument("--max-neighbours", type=int, default=None,
                    help="single and large scenes: neighbour-list capacity (default: the scene's)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.steps is None:
        args.steps = {"batch": 300, "large": 200}.get(args.workload, 500)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "aux":
        return run_aux(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
