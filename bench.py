"""Benchmark: Warren1995 Ni-Cu solidification, 2-D 1024x1024 FP32 (phi, c),
engine-default parameters, dx = 4.6e-8 m, solid disk r = 5 cells at the
centre, c = 0.40783 + U(-1e-3, 1e-3) (seed 0), no-flux boundaries, noise
alpha = 0.3 from the Philox stream; one bench step = 10,000 time steps.

Metric: cell-updates/s (one cell advanced one time step, both fields).
  value  device-resident throughput (fields already in HBM), CUDA events on
         the engine's stream, summed over the K timed bench steps; before
         each bench step the seeded state is restored on the device and L2
         is flushed (a 256 MiB write), outside the events, so every step is
         the same 10,000 steps from the initial state.
  e2e    the same metric through the engine's public API from host numpy
         fields: send_fields_to_GPU (pinned H2D) + simulate(10000) +
         retrieve_fields_from_GPU (D2H), wall clock, per bench step.
  roofline  the Warren1995 step kernel: 16 algorithmic bytes per
         cell-update (read and write phi and c once) x cells per launch /
         average launch-to-launch time, against the measured HBM copy peak.
         The 16 MiB state stays in L2, so this is an effective figure and
         the kernel is bound by FP32 instruction issue and latency:
         issue_frac = warp instructions per launch (the committed ncu
         capture named in `capture`) / (SMs x 4 schedulers x sampled SM
         clock x launch time); traffic = that capture's DRAM bytes.
  fp64   the same workload in float64, device timed (one bench step).
  sweep  three cases beyond L2 (Diffusion 2-D 16384^2, Cahn-Hilliard 3-D
         256^3, Warren1995 4096^2), 100 steps each, CUDA events: the
         HBM-bound kernels' fraction of the copy peak.
  cpu_baseline  the FP64 numpy oracle (oracle/restate.py, a restatement of
         Engines/Warren1995.py:50-92) on a bounded sample of the same
         workload on one host core.

--impl reference times that CPU implementation as the reference arm.
With --gpus N (torchrun, one rank per GPU) every rank runs its own replica:
value = N x per-replica work / max-over-ranks time ("replicas", weak).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SHAPE = (1024, 1024)
SIM_STEPS = 10_000
DX = 4.6e-8
SEED = 0
B_ALG = 16  # bytes per cell-update: phi and c read once and written once (fp32)
METRIC = "cell-updates/s"
WORKLOAD = "warren1995_2d_1024x1024_fp32_10000_steps"


def initial_fields(shape=SHAPE):
    rng = np.random.default_rng(SEED)
    phi = np.ones(shape)
    yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
    phi[(yy - shape[0] // 2) ** 2 + (xx - shape[1] // 2) ** 2 < 25] = 0.0
    c = 0.40783 + rng.uniform(-1e-3, 1e-3, shape)
    return phi, c


def warren_params():
    from oracle import restate
    return dict(restate.WARREN_DEFAULTS, alpha=0.3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_capture():
    """The ncu capture of one Warren1995 launch on the benchmark grid
    (profiles/warren1995_1024_ncu.json: DRAM bytes and warp instructions per
    launch, with the command that made it). Counters cannot be read without
    a profiler, so the bench line quotes the capture and names it."""
    p = ROOT / "profiles" / "warren1995_1024_ncu.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        import tempfile
        out = os.environ.get("PPF_CLOCKS_DIR", tempfile.gettempdir())
        self.path = Path(out) / f"ppf_clocks_rank{index}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return self
        # nvidia-smi takes a moment to start: wait (bounded) for its first
        # sample so that a short timed region is still covered by samples
        t_end = time.perf_counter() + 5.0
        while time.perf_counter() < t_end and self.proc.poll() is None:
            self.f.flush()
            if self.path.stat().st_size > 0:
                break
            time.sleep(0.05)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return None
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[3:7]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r)
                          if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def cpu_baseline(shape=SHAPE, steps=None, budget_s=15.0):
    """FP64 numpy oracle on one core, bounded sample of the workload."""
    from oracle import restate
    phi, c = initial_fields(shape)
    p = warren_params()
    restate.run_warren(phi, c, 1, "NEUMANN", DX, p, seed=SEED)  # warm-up
    t0 = time.perf_counter()
    n = 0
    while True:
        restate.run_warren(phi, c, 1, "NEUMANN", DX, p, seed=SEED, step0=n)
        n += 1
        el = time.perf_counter() - t0
        if (steps is not None and n >= steps) or (steps is None and el > budget_s):
            break
    rate = shape[0] * shape[1] * n / el
    return {"value": rate, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": f"{n} steps of Warren1995 {shape[0]}x{shape[1]} FP64 numpy oracle "
                      f"(alpha=0.3), {el:.1f} s, 1 thread"}


def _reference_sample(args):
    """One worker of the reference arm: `steps` bench steps of `per_step`
    time steps of the benchmark workload (FP64 numpy restatement)."""
    steps, per_step, warmup = args
    from oracle import restate
    phi, c = initial_fields()
    p = warren_params()
    for _ in range(warmup):
        restate.run_warren(phi, c, 1, "NEUMANN", DX, p, seed=SEED)
    t0 = time.perf_counter()
    for k in range(steps):
        restate.run_warren(phi, c, per_step, "NEUMANN", DX, p, seed=SEED, step0=k * per_step)
    return time.perf_counter() - t0


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    # bounded sample per bench step: a few time steps of the same workload,
    # run by one worker process per host core (numpy steps one grid on one
    # thread, so the host's cores are used as independent replicas)
    per_step = max(1, int(os.environ.get("PPF_REF_STEPS", "4")))
    workers = max(1, int(os.environ.get("PPF_REF_WORKERS", str(os.cpu_count() or 1))))
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(workers) as pool:
        times = pool.map(_reference_sample, [(args.steps, per_step, max(args.warmup, 0))] * workers)
    el = max(times)
    wall = time.perf_counter() - t0
    rate = workers * SHAPE[0] * SHAPE[1] * per_step * args.steps / el
    line = {"metric": METRIC, "value": rate, "unit": "cell-updates/s", "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_steps_per_bench_step": per_step,
                       "implementation": "FP64 numpy restatement of Engines/Warren1995.py:50-92",
                       "workers": workers, "wall_s": wall},
            "cpu_baseline": {"value": rate, "unit": METRIC, "cores": workers, "kind": "port",
                             "sample": f"{per_step} time steps per bench step at 1024x1024 on each "
                                       f"of {workers} worker processes (one per host core), "
                                       "time = slowest worker"},
            "e2e": {"value": rate, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def make_sim(phi, c, graph_chunk, precision="fp32"):
    from pyphasefield_gb300 import Warren1995GB300
    sim = Warren1995GB300(dimensions=list(SHAPE), dx=DX, boundary_conditions="NEUMANN",
                          user_data={"seed": SEED, "alpha": 0.3, "graph_chunk": graph_chunk,
                                     "precision": precision})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = phi
    sim.fields[1].data[1:-1, 1:-1] = c
    return sim


def run_gb300(args):
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    import __graft_entry__
    if not (ROOT / "pyphasefield_gb300" / "libppf_gb300.so").exists():
        __graft_entry__.build()

    phi0, c0 = initial_fields()
    chunk = args.graph_chunk
    sim = make_sim(phi0, c0, chunk)
    sim._begun_simulation = True
    sim.just_before_simulating()  # set-up and upload of the seeded state
    stream = sim._ppf_stream
    with torch.cuda.stream(stream):
        init = [t.clone() for t in sim._ppf_bufs[sim._ppf_cur]]
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")

    def restart():
        """Every bench step advances the seeded state by sim_steps from step
        0 (the same work and noise stream each time); restored on the device
        and followed by an L2 flush, outside the timed region."""
        with torch.cuda.stream(stream):
            for t, i in zip(sim._ppf_bufs[sim._ppf_cur], init):
                t.copy_(i)
            flush.fill_(1.0)
        sim.time_step_counter = 0

    for _ in range(args.warmup):  # the first also captures the CUDA graph
        restart()
        sim.simulate(args.sim_steps)
    sim.synchronize()

    cells = SHAPE[0] * SHAPE[1]
    events = []
    barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            restart()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sim.simulate(args.sim_steps)
            e1.record(stream)
            events.append((e0, e1))
        torch.cuda.synchronize()
        barrier()
    wall = time.perf_counter() - wall0
    dev_s = sum(a.elapsed_time(b) for a, b in events) / 1e3
    dev_s = max_over_ranks(dev_s)
    work = cells * args.sim_steps * args.steps
    value = world * work / dev_s
    step_launch_s = dev_s / (args.steps * args.sim_steps)

    # e2e through the public API with host fields, per bench step: new host
    # fields -> send_fields_to_GPU (pinned H2D) -> simulate -> retrieve (D2H)
    e2e_times = []
    h2d = d2h = 2 * cells * 4
    sim2 = make_sim(phi0, c0, chunk)
    sim2.simulate(chunk)  # one-time set-up (buffers, graph capture) outside timing
    sim2.retrieve_fields_from_GPU()
    for k in range(args.e2e_steps):
        sim2.fields[0].data[1:-1, 1:-1] = phi0
        sim2.fields[1].data[1:-1, 1:-1] = c0
        barrier()
        t0 = time.perf_counter()
        sim2.send_fields_to_GPU()
        sim2.simulate(args.sim_steps)
        sim2.retrieve_fields_from_GPU()
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.mean(e2e_times)))
    e2e_value = world * cells * args.sim_steps / e2e_s

    # the same workload in float64 (the precision of the reference), device
    # timed: one warm-up and one timed bench step
    fp64 = None
    if not args.no_fp64:
        sim64 = make_sim(phi0, c0, chunk, precision="fp64")
        sim64._begun_simulation = True
        sim64.just_before_simulating()
        s64 = sim64._ppf_stream
        with torch.cuda.stream(s64):
            init64 = [t.clone() for t in sim64._ppf_bufs[sim64._ppf_cur]]
        sims64 = []
        for k in range(2):
            with torch.cuda.stream(s64):
                for t, i in zip(sim64._ppf_bufs[sim64._ppf_cur], init64):
                    t.copy_(i)
                flush.fill_(1.0)
            sim64.time_step_counter = 0
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(s64)
            sim64.simulate(args.sim_steps)
            b.record(s64)
            b.synchronize()
            sims64.append(a.elapsed_time(b) / 1e3)
        sec64 = max_over_ranks(sims64[-1])
        fp64 = {"value": world * cells * args.sim_steps / sec64, "unit": METRIC,
                "ms_per_step": 1e3 * sec64, "dtype": "f64",
                "kernel": "warren1995_kernel<double>",
                "per_launch_us": sec64 / args.sim_steps * 1e6}
        del sim64, init64

    sweep = None
    if not args.no_sweep:
        sweep = {}
        for name, steps in (("diffusion_16384", 100), ("cahn_hilliard_256", 100),
                            ("warren1995_4096", 100)):
            sweep[name] = time_sweep_case(name, steps)
            torch.cuda.empty_cache()

    if rank == 0:
        peak, peak_kind = peaks()
        achieved = B_ALG * cells / step_launch_s / 1e9
        cap = committed_capture()
        # per graph chunk: the steps, the step counter, and the status watch
        # (NaN/Inf sentinel per field and the status collect)
        n_chunks = -(-args.sim_steps // chunk)
        launches = args.steps * (args.sim_steps + n_chunks * (1 + sim._ppf_watch_launches()))
        sm_count = torch.cuda.get_device_properties(local).multi_processor_count
        line = {
            "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "global_batch": world, "time_steps_per_step":
                       args.sim_steps, "grid": list(SHAPE), "alpha": 0.3,
                       "parallelism": f"replicas{world}",
                       "l2": "flushed between bench steps (256 MiB write); the 16 MiB "
                             "double-buffered state is L2-resident within a step",
                       "graph_chunk": chunk},
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "L2-resident state; FP32 issue/latency",
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": cap.get("dram_bytes_per_launch"),
                         "peak_source": peak_kind,
                         "kernel": cap.get("kernel", "warren1995_f2_kernel"),
                         "per_launch_us": step_launch_s * 1e6},
            "gpu_launches": launches,
            "wall_s": wall,
        }
        clocks = clk.summary()
        if clocks:
            line["clocks"] = clocks
        if cap.get("warp_instructions_per_launch"):
            # warp instructions issued per launch (ncu) over the issue slots of
            # the average launch: SMs x 4 schedulers x SM clock x launch time
            mhz = (clocks or {}).get("sm_mhz") or cap.get("sm_mhz")
            slots = sm_count * 4 * mhz * 1e6 * step_launch_s
            line["roofline"]["issue_frac"] = cap["warp_instructions_per_launch"] / slots
            line["roofline"]["capture"] = cap.get("source")
        if fp64:
            line["fp64"] = fp64
        if sweep:
            line["sweep"] = sweep
        if not args.no_cpu_baseline and world == 1:  # the CPU baseline is an N = 1 figure
            line["cpu_baseline"] = cpu_baseline(budget_s=args.cpu_budget)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


SWEEP = {
    # name: (model, grid, temporal depth, steps); grids exceed the 129 MB L2
    "diffusion_4096": ("diffusion", (4096, 4096), 1, 200),
    "diffusion_8192": ("diffusion", (8192, 8192), 1, 100),
    "diffusion_16384": ("diffusion", (16384, 16384), 1, 100),
    "diffusion_8192_d4": ("diffusion", (8192, 8192), 4, 200),
    "diffusion_16384_d4": ("diffusion", (16384, 16384), 4, 100),
    "diffusion_16384_d8": ("diffusion", (16384, 16384), 8, 200),
    "diffusion_16384_d2": ("diffusion", (16384, 16384), 2, 100),
    "diffusion_8192_d8": ("diffusion", (8192, 8192), 8, 200),
    "allen_cahn_16384_d8": ("allen_cahn", (16384, 16384), 8, 200),
    "diffusion_16384_d4_fp64": ("diffusion", (16384, 16384), 4, 100, {"precision": "fp64"}),
    "diffusion_16384_d8_seg512": ("diffusion", (16384, 16384), 8, 200, {"tile": (0, 512)}),
    "diffusion_16384_d4_seg256": ("diffusion", (16384, 16384), 4, 100, {"tile": (0, 256)}),
    "allen_cahn_4096": ("allen_cahn", (4096, 4096), 1, 200),
    "allen_cahn_8192": ("allen_cahn", (8192, 8192), 1, 100),
    "allen_cahn_16384": ("allen_cahn", (16384, 16384), 1, 100),
    "allen_cahn_16384_d4": ("allen_cahn", (16384, 16384), 4, 100),
    "warren1995_4096": ("warren1995", (4096, 4096), 1, 100),
    "warren1995_8192": ("warren1995", (8192, 8192), 1, 100),
    # every cell takes the full update (no exact bulk shortcut): the cost of
    # a grid that is interface everywhere
    "warren1995_4096_full": ("warren1995", (4096, 4096), 1, 100, {"bulk_shortcut": False}),
    "diffusion3d_384": ("diffusion", (384, 384, 384), 1, 100),
    "diffusion3d_512": ("diffusion", (512, 512, 512), 1, 100),
    "allen_cahn3d_512": ("allen_cahn", (512, 512, 512), 1, 100),
    "cahn_hilliard_256": ("cahn_hilliard", (256, 256, 256), 1, 500),
    "cahn_hilliard_384": ("cahn_hilliard", (384, 384, 384), 1, 100),
    "cahn_hilliard_512": ("cahn_hilliard", (512, 512, 512), 1, 100),
    "ensemble_64": ("ensemble", None, 1, 2000),
    # the same 64 members stepped one after another, each as its own engine
    # (its own kernel launches and CUDA graphs): what batching saves
    "ensemble_64_solo": ("ensemble_solo", None, 1, 2000),
    # implicit / Crank-Nicolson diffusion (periodic line solves or the full
    # system), D dt / dx^2 = 5
    "implicit_adi_8192": ("diffusion", (8192, 8192), 1, 50,
                          {"solver": "implicit", "adi": True, "dt": 5.0}),
    "crank_nicolson_adi_8192": ("diffusion", (8192, 8192), 1, 50,
                                {"solver": "crank-nicolson", "adi": True, "dt": 5.0}),
    "implicit_adi3d_512": ("diffusion", (512, 512, 512), 1, 20,
                           {"solver": "implicit", "adi": True, "dt": 5.0}),
    "crank_nicolson_adi3d_512": ("diffusion", (512, 512, 512), 1, 20,
                                 {"solver": "crank-nicolson", "adi": True, "dt": 5.0}),
    "implicit_full_4096": ("diffusion", (4096, 4096), 1, 5,
                           {"solver": "implicit", "adi": False, "dt": 5.0}),
    # semi-implicit Allen-Cahn (a diagonal that varies per cell): M eps^2 dt / dx^2 = 0.1,
    # 16 W M dt = 1.6
    "allen_cahn_implicit_adi_8192": ("allen_cahn", (8192, 8192), 1, 50,
                                     {"solver": "implicit", "adi": True, "dt": 1.0}),
    "allen_cahn_cn_adi_8192": ("allen_cahn", (8192, 8192), 1, 50,
                               {"solver": "crank-nicolson", "adi": True, "dt": 1.0}),
    "allen_cahn_implicit_adi3d_512": ("allen_cahn", (512, 512, 512), 1, 20,
                                      {"solver": "implicit", "adi": True, "dt": 1.0}),
    "allen_cahn_full_4096": ("allen_cahn", (4096, 4096), 1, 5,
                             {"solver": "implicit", "adi": False, "gmres": True, "dt": 1.0}),
    # NCGPU (Ni-Cu, 1574 K, one seed at the centre, dx = 4.6e-6 cm): float64 (the engine's
    # default) and float32
    "ncgpu_2048": ("ncgpu", (2048, 2048), 1, 100, {"precision": "fp64"}),
    "ncgpu_2048_fp32": ("ncgpu", (2048, 2048), 1, 100, {"precision": "fp32"}),
    # six components (Ni-Cu-Al and three pseudo-elements): five concentration fields
    "ncgpu_6comp_2048": ("ncgpu", (2048, 2048), 1, 50,
                         {"precision": "fp64", "tdb": "ncgpu_6comp.tdb",
                          "c0": [0.05, 0.2, 0.3, 0.1, 0.15]}),
    # Ni-Nb with binary Redlich-Kister terms (the reference's non-ideal database), and the
    # NCGPU_new variant (per-component derivatives and noise, phase and orientation noise)
    "ncgpu_ninb_2048": ("ncgpu", (2048, 2048), 1, 50,
                        {"precision": "fp64", "tdb": "ncgpu_ninb.tdb", "c0": [0.1]}),
    "ncgpu_new_2048": ("ncgpu_new", (2048, 2048), 1, 50, {"precision": "fp64"}),
}
SWEEP_B_ALG = {"diffusion": 8, "allen_cahn": 8, "cahn_hilliard": 8, "warren1995": 16}
NCGPU_TDB = ROOT / "tests" / "golden" / "ncgpu_nicu.tdb"


def sweep_engine(model, grid, depth, steps, rng, extra=None):
    """An engine of `model` on `grid` with seeded synthetic fields."""
    from pyphasefield_gb300 import (CahnAllenGB300, CahnHilliardGB300, DiffusionGB300,
                                    Warren1995GB300)
    extra = dict(extra or {})
    dt = extra.pop("dt", None)
    ud = dict({"graph_chunk": min(steps, 100), "temporal_depth": depth}, **extra)
    if model == "diffusion":
        sim = DiffusionGB300(dimensions=list(grid), dx=1.0, dt=dt or 0.2,
                             boundary_conditions="PERIODIC", user_data=dict(ud, D=1.0))
        init = [0.5 + 0.01 * rng.standard_normal(grid)]
    elif model == "allen_cahn":
        sim = CahnAllenGB300(dimensions=list(grid), dx=1.0, dt=dt or 0.1,
                             boundary_conditions="NEUMANN", user_data=dict(ud))
        init = [rng.random(grid)]
    elif model == "cahn_hilliard":
        sim = CahnHilliardGB300(dimensions=list(grid), dx=1.0, dt=0.01,
                                boundary_conditions="PERIODIC",
                                user_data=dict(ud, M=1.0, epsilon=1.0))
        init = [0.5 + rng.uniform(-0.05, 0.05, grid)]
    elif model in ("ncgpu", "ncgpu_new"):
        from pyphasefield_gb300 import NCGPU_newGB300, NCGPUGB300
        tdb = NCGPU_TDB.parent / ud.pop("tdb", NCGPU_TDB.name)
        c0 = ud.pop("c0", [0.40831])
        cls = NCGPUGB300 if model == "ncgpu" else NCGPU_newGB300
        sim = cls(dimensions=list(grid), dx=4.6e-6, tdb_path=str(tdb),
                         temperature_type="ISOTHERMAL", initial_T=1574.0,
                         boundary_conditions="PERIODIC",
                         user_data=dict(ud, sim_type="seed", initial_concentration_array=c0,
                                        seed=SEED))
        sim.initialize_fields_and_imported_data()
        return sim
    else:
        sim = Warren1995GB300(dimensions=list(grid), dx=DX, boundary_conditions="NEUMANN",
                              user_data=dict(ud, seed=SEED, alpha=0.3))
        phi, c = initial_fields(grid)
        init = [phi, c]
    sim.initialize_fields_and_imported_data()
    sl = (slice(1, -1),) * len(grid)
    for f, v in zip(sim.fields, init):
        f.data[sl] = v
    return sim


def sweep_bytes_per_cell(model, sim) -> int:
    """Algorithmic bytes per cell and step: every field read and written once
    per step; for the implicit solvers once per line sweep (ADI: one sweep per
    axis) or per Chebyshev iteration (iterate, previous iterate and the
    right-hand side read, the new iterate written: 16 B in float)."""
    ud = sim.user_data
    if model in ("ncgpu", "ncgpu_new"):
        # phi, q1, q4 and every concentration field read and written, the
        # temperature read
        return (2 * len(sim.fields) + 1) * (8 if ud.get("precision", "fp64") == "fp64" else 4)
    if model in ("diffusion", "allen_cahn") and ud.get("solver", "explicit") != "explicit":
        if ud.get("adi") or len(sim.dimensions) == 1:
            return 8 * len(sim.dimensions)
        return 16 * sim._ppf_iterations
    return SWEEP_B_ALG[model]


def run_sweep(args):
    """Roofline sweep at sizes beyond L2 (plus the Cahn-Hilliard 256^3 and
    64-member ensemble workloads): one JSON line per case."""
    import torch
    import __graft_entry__
    if not (ROOT / "pyphasefield_gb300" / "libppf_gb300.so").exists():
        __graft_entry__.build()
    names = list(SWEEP) if args.sweep == "all" else args.sweep.split(",")
    for name in names:
        print(json.dumps(time_sweep_case(name)), flush=True)
        torch.cuda.empty_cache()


def time_sweep_case(name, steps=None):
    """One sweep case: set-up, upload and warm-up (with graph capture), then
    `steps` steps (default: the case's own) timed with CUDA events on the
    engine's stream. Returns the case's JSON record."""
    import torch
    peak, peak_kind = peaks()
    model, grid, depth, case_steps = SWEEP[name][:4]
    steps = steps or case_steps
    extra = SWEEP[name][4] if len(SWEEP[name]) > 4 else None
    rng = np.random.default_rng(0)
    if model == "ensemble_solo":
        from pyphasefield_gb300.ensemble import make_config_ensemble
        sims = make_config_ensemble(n=64, seed=0, graph_chunk=100)
        for sm in sims:
            sm.simulate(100)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for sm in sims:
            sm.simulate(steps)
            sm.synchronize()
        sec = time.perf_counter() - t0
        cells = sum(sm._ppf_grid.cells for sm in sims)
        byts = sum(sm._ppf_grid.cells * (16 if len(sm.fields) == 2 else 8) for sm in sims)
        del sims
        return {"sweep": name, "model": model, "grid": "config ensemble, members alone",
                "steps": steps, "cells": cells, "cell_updates_per_s": cells * steps / sec,
                "ms_per_step": 1e3 * sec / steps, "algorithmic_bytes_per_step": byts,
                "achieved_gbs": byts * steps / sec / 1e9, "peak_gbs": peak,
                "peak_source": peak_kind, "frac": byts * steps / sec / 1e9 / peak,
                "timing": "host wall clock, members one after another"}
    if model == "ensemble":
        from pyphasefield_gb300.ensemble import Ensemble, make_config_ensemble
        sims = make_config_ensemble(n=64, seed=0)
        runner = Ensemble(sims, graph_chunk=100)
        cells = runner.cells
        bytes_per_step = sum(s._ppf_grid.cells * (16 if len(s.fields) == 2 else 8)
                             for s in sims)
        stream = runner.stream
        advance = runner.simulate
    else:
        sim = sweep_engine(model, grid, depth, steps, rng, extra)
        cells = int(np.prod(grid))
        advance = sim.simulate
    advance(min(steps, 100))  # set-up, upload, graph capture, warm-up
    if model != "ensemble":
        bytes_per_step = sweep_bytes_per_cell(model, sim) * cells
    if model != "ensemble":
        stream = sim._ppf_stream
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record(stream)
        advance(steps)
        e1.record(stream)
        e1.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    line = {"sweep": name, "model": model, "grid": list(grid) if grid else "config ensemble",
            "temporal_depth": depth, "steps": steps, "cells": cells, "options": extra or {},
            "cell_updates_per_s": cells * steps / sec, "ms_per_step": 1e3 * sec / steps,
            "algorithmic_bytes_per_step": bytes_per_step,
            "achieved_gbs": bytes_per_step * steps / sec / 1e9, "peak_gbs": peak,
            "peak_source": peak_kind}
    line["frac"] = line["achieved_gbs"] / peak
    # SM clocks sampled every 200 ms during the timed steps (null when
    # the case ends before the first sample)
    line["clocks"] = clk.summary()
    if model == "cahn_hilliard":
        m = sim.collect_mass_history()
        line["mass_rel_drift"] = float(abs(m[-1] - m[0]) / abs(m[0]))
    del advance, stream
    if model == "ensemble":
        del runner, sims
    else:
        del sim
    return line


def _errors(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return {"rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
            "linf": float(np.abs(a - b).max())}


def run_accuracy(args):
    """FP32 engines against FP64 references per configuration, one JSON
    line each: Diffusion 256^2 against the numpy oracle (oracle/restate.py,
    the reference's own engine functions restated), Warren1995 1024^2,
    Cahn-Hilliard 256^3 and ensemble members against the FP64 engines (the
    same kernels in double, equal to the oracle within 1e-12 in the tests)."""
    import __graft_entry__
    from oracle import restate
    from pyphasefield_gb300 import DiffusionGB300
    if not (ROOT / "pyphasefield_gb300" / "libppf_gb300.so").exists():
        __graft_entry__.build()
    rng = np.random.default_rng(SEED)

    def cells(sim):
        sim.retrieve_fields_from_GPU()
        return [f.get_cells().copy() for f in sim.fields]

    # configuration 1: Diffusion 2-D 256^2, dt = 0.2, periodic, 1000 steps
    c0 = 0.5 + 0.01 * rng.standard_normal((256, 256))
    sim = DiffusionGB300(dimensions=[256, 256], dx=1.0, dt=0.2, boundary_conditions="PERIODIC",
                         user_data={"D": 1.0})
    sim.initialize_fields_and_imported_data()
    sim.fields[0].data[1:-1, 1:-1] = c0
    sim.simulate(1000)
    ref = restate.run_single("diffusion", c0, 1000, "PERIODIC", 1.0, 0.2, D=1.0)
    print(json.dumps({"accuracy": "diffusion_256_1000", "reference": "fp64 numpy oracle",
                      "c": _errors(cells(sim)[0], ref)}), flush=True)

    # configuration 2: Warren1995 1024^2, alpha = 0 (parity run), 1000 and 10,000 steps
    phi0, cc0 = initial_fields()
    _warren_accuracy(phi0, cc0, cells, "")
    # the same with the disk centred between cells (511.5, 511.5): no cell
    # sits at the seed's centre, where grad phi = 0 exactly and the angle
    # is set by rounding residue (atan2 of two FP64 residues)
    yy, xx = np.mgrid[0:SHAPE[0], 0:SHAPE[1]]
    phi_h = np.ones(SHAPE)
    phi_h[(yy - 511.5) ** 2 + (xx - 511.5) ** 2 < 25] = 0.0
    _warren_accuracy(phi_h, cc0, cells, "_offcentre")
    _rest_of_accuracy(rng, cells)


def _warren_accuracy(phi0, cc0, cells, tag):
    from pyphasefield_gb300 import Warren1995GB300
    runs = {}
    for prec in ("fp32", "fp64"):
        w = Warren1995GB300(dimensions=list(SHAPE), dx=DX, boundary_conditions="NEUMANN",
                            user_data={"seed": SEED, "alpha": 0.0, "precision": prec})
        w.initialize_fields_and_imported_data()
        w.fields[0].data[1:-1, 1:-1] = phi0
        w.fields[1].data[1:-1, 1:-1] = cc0
        w.simulate(1000)
        a = cells(w)
        w.simulate(9000)
        runs[prec] = (a, cells(w))
    for i, n in enumerate((1000, 10000)):
        print(json.dumps({"accuracy": f"warren1995_1024_{n}{tag}", "reference": "fp64 engine",
                          "alpha": 0.0,
                          "phi": _errors(runs["fp32"][i][0], runs["fp64"][i][0]),
                          "c": _errors(runs["fp32"][i][1], runs["fp64"][i][1])}), flush=True)


def _rest_of_accuracy(rng, cells):
    import torch
    from pyphasefield_gb300 import CahnHilliardGB300
    # configuration 3: Cahn-Hilliard 3-D 256^3, dt = 0.01, periodic, 1000 steps
    u0 = 0.5 + rng.uniform(-0.05, 0.05, (256, 256, 256))
    out = {}
    for prec in ("fp32", "fp64"):
        ch = CahnHilliardGB300(dimensions=[256, 256, 256], dx=1.0, dt=0.01,
                               boundary_conditions="PERIODIC",
                               user_data={"M": 1.0, "epsilon": 1.0, "precision": prec})
        ch.initialize_fields_and_imported_data()
        ch.fields[0].data[1:-1, 1:-1, 1:-1] = u0
        ch.simulate(1000)
        m = ch.collect_mass_history()
        out[prec] = (cells(ch)[0], float(abs(m[-1] - m[0]) / abs(m[0])))
        del ch
        torch.cuda.empty_cache()
    print(json.dumps({"accuracy": "cahn_hilliard_256_1000", "reference": "fp64 engine",
                      "c": _errors(out["fp32"][0], out["fp64"][0]),
                      "mass_rel_drift_fp32": out["fp32"][1],
                      "mass_rel_drift_fp64": out["fp64"][1]}), flush=True)

    # configuration 4: ensemble members (fp32, one launch per step) against
    # the same members stepped alone in fp64, 2000 steps (first 8 members)
    from pyphasefield_gb300.ensemble import Ensemble, make_config_ensemble
    ens_sims = make_config_ensemble(n=64, seed=0)[:8]
    solo = make_config_ensemble(n=64, seed=0, precision="fp64")[:8]
    Ensemble(ens_sims, graph_chunk=100).simulate(2000)
    members = []
    for a, b in zip(ens_sims, solo):
        b.simulate(2000)
        m = {"model": type(a).__name__, "side": int(a.dimensions[0])}
        for name, fa, fb in zip(("phi", "c"), cells(a), cells(b)):
            e = _errors(fa, fb)
            if not np.linalg.norm(fb) > 1e-6 * np.sqrt(fb.size):  # field gone to ~0
                e = {"rms": float(np.sqrt(np.mean((fa - fb) ** 2))), "linf": e["linf"]}
            m[name] = e
        members.append(m)
    print(json.dumps({"accuracy": "ensemble_members_2000", "reference": "fp64 engines, alone",
                      "alpha": 0.3, "members": members}), flush=True)


def profile_case(name: str):
    """Small eager workloads (no timing, no graphs) for ncu captures:
    warren1024  the benchmark grid, 2005 steps (capture launch 2002: a grown crystal)
    warren1024_late  the benchmark grid, 9605 steps (capture launch 9600: the state the
                last tenth of a bench step runs on; no cell is exactly bulk any more)
    ch256       Cahn-Hilliard 256^3 periodic, dt 0.01, 5 steps
    diff4096    Diffusion 2-D 4096^2 periodic, 5 steps (temporal depth from PPF_DEPTH, default 1)
    diff3d384   Diffusion 3-D 384^3 periodic, 5 steps
    ensemble64  the 64-member ensemble benchmark (1.56e7 cells), two rows and four bands per
                warp: 40 steps, one launch each
    ensemble64_tall  the same with four rows and four bands per warp, per-step launches (the
                autotuner's choice for this mix): 40 steps
    warren4096  Warren1995 4096^2 from the sweep's seeded state, 5 steps (the engines' default
                of eight rows per warp at this size)
    tb4096      Diffusion 2-D 4096^2, depth 4 on 128 x 32 shared-memory tiles, 20 steps
    reduce4096  five FP64 sums of a 4096^2 float field (ppf_reduce_sum_f32)
    acfull2048  implicit Allen-Cahn, full 2-D system on 2048^2 (Chebyshev), fp64, 2 steps
    acminres1024  the same beyond the Chebyshev bound (16 W M dt = 7.3, an indefinite
                system: MINRES in one persistent launch) on 1024^2, fp64, 2 steps
    surrogate_train  six Adam steps of the default surrogate network on 512^2 stencil
                snapshots, batch 8 (8192 tokens): the tcgen05 and mma.sync GEMMs, the
                depthwise convolutions
    diff8192    Diffusion 2-D 8192^2 periodic, 5 passes of PPF_DEPTH (default 4) steps: the
                marching temporal-blocking kernel on 512 MiB of fields
    diff16384   Diffusion 2-D 16384^2 periodic, 5 steps (2 GiB of fields: beyond L2)
    adi4096     implicit ADI Diffusion 2-D 4096^2 (Crank-Nicolson with PPF_CN=1), D dt = 5,
                3 steps: line solves along x and y
    acadi4096   semi-implicit ADI Allen-Cahn 2-D 4096^2, dt = 1, 3 steps: variable-diagonal
                line solves along x and y
    ncgpu1024   NCGPU Ni-Cu 1024^2 (precision from PPF_PRECISION, default fp64), 5 steps
    """
    import torch
    from pyphasefield_gb300 import CahnHilliardGB300, DiffusionGB300
    rng = np.random.default_rng(0)
    if name in ("warren1024", "warren1024_late"):
        phi0, c0 = initial_fields()
        sim = make_sim(phi0, c0, 100)
        sim.user_data["use_graph"] = False
        sim.simulate(2005 if name == "warren1024" else 9605)
    elif name == "ch256":
        sim = CahnHilliardGB300(dimensions=[256, 256, 256], dx=1.0, dt=0.01,
                                boundary_conditions="PERIODIC",
                                user_data={"M": 1.0, "epsilon": 1.0, "use_graph": False})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1, 1:-1] = 0.5 + rng.uniform(-0.05, 0.05, (256, 256, 256))
        sim.simulate(5)
    elif name == "diff4096":
        depth = int(os.environ.get("PPF_DEPTH", "1"))
        sim = DiffusionGB300(dimensions=[4096, 4096], dx=1.0, dt=0.2,
                             boundary_conditions="PERIODIC",
                             user_data={"D": 1.0, "use_graph": False, "temporal_depth": depth})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1] = 0.5 + 0.01 * rng.standard_normal((4096, 4096))
        sim.simulate(5 * depth)
    elif name in ("ensemble64", "ensemble64_tall"):
        from pyphasefield_gb300.ensemble import Ensemble, make_config_ensemble
        rows = 2 if name == "ensemble64" else 4
        ens = Ensemble(make_config_ensemble(n=64, seed=0), rows=rows, bands=4, graph_chunk=8,
                       use_graph=False, persistent=False)
        ens.simulate(40)
        ens.synchronize()
        return
    elif name == "warren4096":
        sim = sweep_engine("warren1995", (4096, 4096), 1, 5, rng, {"use_graph": False})
        sim.simulate(5)
    elif name == "tb4096":
        sim = DiffusionGB300(dimensions=[4096, 4096], dx=1.0, dt=0.2,
                             boundary_conditions="PERIODIC",
                             user_data={"D": 1.0, "use_graph": False, "temporal_depth": 4,
                                        "tile": (128, 32)})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1] = 0.5 + 0.01 * rng.standard_normal((4096, 4096))
        sim.simulate(20)
    elif name == "reduce4096":
        import ctypes as C
        from pyphasefield_gb300 import _lib as L
        from pyphasefield_gb300.device import DeviceGrid
        g = DeviceGrid((4096, 4096), torch.float32, torch.device("cuda"))
        x = g.empty()
        x.uniform_()
        n = C.c_size_t()
        L.call("ppf_reduce_scratch_bytes", C.byref(g.grid), C.byref(n))
        scratch = torch.empty(n.value, dtype=torch.uint8, device="cuda")
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        for _ in range(5):
            L.call("ppf_reduce_sum_f32", C.c_void_p(x.data_ptr()), C.byref(g.grid),
                   C.c_void_p(out.data_ptr()), C.c_void_p(scratch.data_ptr()), n, sp)
    elif name in ("acfull2048", "acminres1024"):
        from pyphasefield_gb300 import CahnAllenGB300
        n = 2048 if name == "acfull2048" else 1024
        full = name == "acfull2048"
        sim = CahnAllenGB300(dimensions=[n, n], dx=1.0 if full else 3.0, dt=1.0 if full else 0.5,
                             boundary_conditions="PERIODIC",
                             user_data={"use_graph": False, "solver": "implicit", "adi": False,
                                        "gmres": True, "M": 0.1 if full else 0.7,
                                        "W": 1.0 if full else 1.3,
                                        "epsilon": 1.0 if full else 1.1, "precision": "fp64"})
        sim.initialize_fields_and_imported_data()
        if full:
            sim.fields[0].data[1:-1, 1:-1] = rng.random((n, n))
        else:  # half the cells at phi = 0.75: an indefinite system (MINRES)
            sim.fields[0].data[1:-1, 1:-1] = np.where(rng.random((n, n)) > 0.5, 0.75, 0.2)
        sim.simulate(2)
    elif name == "surrogate_train":
        from pyphasefield_gb300 import surrogate as S
        data = S.generate_trajectories(2, 512, 64, 16, seed=1, warm_steps=16)
        net = S.SurrogateNet(seed=0)
        net.fit_normalisation(data, 512)
        S.train(net, data, 512, iters=6, batch=8, log_every=1000)
    elif name == "diff8192":
        depth = int(os.environ.get("PPF_DEPTH", "4"))
        sim = DiffusionGB300(dimensions=[8192, 8192], dx=1.0, dt=0.2,
                             boundary_conditions="PERIODIC",
                             user_data={"D": 1.0, "use_graph": False, "temporal_depth": depth})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1] = 0.5 + 0.01 * rng.standard_normal((8192, 8192))
        sim.simulate(5 * depth)
    elif name == "diff16384":
        sim = DiffusionGB300(dimensions=[16384, 16384], dx=1.0, dt=0.2,
                             boundary_conditions="PERIODIC", user_data={"D": 1.0, "use_graph": False})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1] = 0.5 + 0.01 * rng.standard_normal((16384, 16384))
        sim.simulate(5)
    elif name == "adi4096":
        solver = "crank-nicolson" if os.environ.get("PPF_CN") == "1" else "implicit"
        sim = DiffusionGB300(dimensions=[4096, 4096], dx=1.0, dt=5.0,
                             boundary_conditions="PERIODIC",
                             user_data={"D": 1.0, "use_graph": False, "solver": solver,
                                        "adi": True})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1] = rng.random((4096, 4096))
        sim.simulate(3)
    elif name == "acadi4096":
        from pyphasefield_gb300 import CahnAllenGB300
        sim = CahnAllenGB300(dimensions=[4096, 4096], dx=1.0, dt=1.0,
                             boundary_conditions="PERIODIC",
                             user_data={"use_graph": False, "solver": "implicit", "adi": True})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1] = rng.random((4096, 4096))
        sim.simulate(3)
    elif name == "ncgpu1024":
        from pyphasefield_gb300 import NCGPUGB300
        sim = NCGPUGB300(dimensions=[1024, 1024], dx=4.6e-6, tdb_path=str(NCGPU_TDB),
                         temperature_type="ISOTHERMAL", initial_T=1574.0,
                         boundary_conditions="PERIODIC",
                         user_data={"use_graph": False, "sim_type": "seed",
                                    "initial_concentration_array": [0.40831],
                                    "precision": os.environ.get("PPF_PRECISION", "fp64")})
        sim.initialize_fields_and_imported_data()
        sim.simulate(5)
    elif name == "diff3d384":
        sim = DiffusionGB300(dimensions=[384, 384, 384], dx=1.0, dt=0.1,
                             boundary_conditions="PERIODIC", user_data={"D": 1.0, "use_graph": False})
        sim.initialize_fields_and_imported_data()
        sim.fields[0].data[1:-1, 1:-1, 1:-1] = 0.5 + 0.01 * rng.standard_normal((384, 384, 384))
        sim.simulate(5)
    else:
        raise SystemExit(f"unknown profile case {name!r}")
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser(description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--profile-case", default=None,
                    help="run a small eager workload for ncu instead of the benchmark")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--sim-steps", type=int, default=SIM_STEPS)
    ap.add_argument("--graph-chunk", type=int, default=500)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the float64 rate of the same workload")
    ap.add_argument("--no-sweep", action="store_true",
                    help="skip the three beyond-L2 cases added to the bench line")
    ap.add_argument("--sweep", default=None,
                    help="roofline sweep instead of the benchmark: 'all' or a comma list of "
                         + ", ".join(SWEEP))
    ap.add_argument("--accuracy", action="store_true",
                    help="FP32 vs FP64 errors per configuration instead of the benchmark")
    args = ap.parse_args()
    if args.accuracy:
        run_accuracy(args)
        return
    if args.sweep:
        run_sweep(args)
        return
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
