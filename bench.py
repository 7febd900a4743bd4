#!/usr/bin/env python
"""bench.py - bubble-substeps/s of the batched bubble step on GB300 (one JSON line on rank 0).

Workload (one "step" = one step of every world of the batch): 4,096 independent worlds (seed 3), bubble counts
log-uniform in [16, 1024], radii U[6, 24] at 40 % area fraction, 0-32 rigid bodies each (polygons, circles, capsules;
half-extents U[8, 40]; static or kinematic), walls, no gravity, dt = 1/60; seeded synthetic data. Defaults: 5 warm-up
and 20 timed steps.

  value        whole-job bubble-substeps/s of the batched path (one persistent launch per step, CUDA graph), inputs
               resident in HBM; device time from CUDA events on the library's stream
  e2e          the same metric through the C ABI with HOST buffers: every step writes (centre, velocity) of all bubbles
               from pinned host memory, steps, and reads them back
  per_world    the plain per-world launch path on the same worlds (one launch per world, one after another)
  latency      p50 / p99 device time of one batched step
  roofline     algorithmic bytes of the dominant kernel (persistent_step_kernel) per second against the measured HBM
               peak
  cpu_baseline the CPU oracle (C++ restatement of the reference's algorithm, OpenMP over worlds, every host thread)
               on the same worlds with the same warm-up and timed steps: the reference arm's own measurement

--impl reference times the reference algorithm on the host cores (the oracle port: the reference itself is Swift +
Metal and cannot run here) on the same worlds, warm-up and timed steps as the GPU arm.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bubble-substeps/s (batched worlds, 1 GB300)"
UNIT = "bubble-substeps/s"
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
PROFILE_FILE = ROOT / "profiles" / "persistent_step_kernel.json"


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def algorithmic_bytes(bubble_substeps: float, bubble_builds: float, mean_degree: float) -> float:
    """Bytes one bubble-substep must move without cache reuse: own state 48 B, constants 28 B, neighbour indices
    4 B x k x 2 passes, neighbour state 16 B x k x 2 passes -> 76 + 40 k; a grid build adds 96 + 8 k per bubble."""
    return bubble_substeps * (76.0 + 40.0 * mean_degree) + bubble_builds * (96.0 + 8.0 * mean_degree)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every POLL_MS ms from start() to stop(); each sample keeps its host
    arrival time so the samples inside a sub-window (the timed steps) can be told apart from the rest."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    POLL_MS = 10  # the timed region of the default run lasts ~40 ms: several samples fall inside it

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[tuple[float, str]] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.POLL_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            deadline = time.time() + 5.0  # the measured window starts once samples flow
            while not self.lines and time.time() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
            self.lines.clear()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def _summary(self, lines) -> dict:
        sm, smax, reasons = [], [], set()
        for _, line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(self.NAMES, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}

    def stop(self, timed: tuple[float, float] | None = None) -> dict:
        """Clocks over the whole window; with `timed` = (t0, t1) host times also the samples taken within it."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        out = self._summary(self.lines)
        if timed is not None:
            inside = self._summary([x for x in self.lines if timed[0] <= x[0] <= timed[1] + self.POLL_MS / 1000.0])
            out["timed_region"] = {"sm_mhz": inside["sm_mhz"], "reasons": inside["reasons"],
                                   "samples": inside["samples"], "seconds": timed[1] - timed[0]}
            out["window"] = f"warm-up, timed steps and end-to-end steps of the batched workload ({self.POLL_MS} ms polling)"
        return out


def pinned_buffer(count: int):
    """A page-locked host buffer of `count` float4 records (torch's pinned allocator; plain numpy otherwise)."""
    try:
        import torch
        t = torch.empty((count, 4), dtype=torch.float32, pin_memory=True)
        return t.numpy(), t
    except Exception:
        a = np.zeros((count, 4), np.float32)
        return a, None


def cpu_leg(specs, steps: int, warmup: int, threads: int = 0) -> dict:
    """The reference's algorithm on the host cores (the C++ oracle port, OpenMP over worlds, every host thread): the
    same worlds, warm-up and timed steps as the GPU arm. Returns bubble-substeps/s over the timed steps."""
    from oracle import oracle
    cores = oracle.set_threads(threads if threads > 0 else (os.cpu_count() or 1))
    worlds = [oracle.OracleWorld(s, 32) for s in specs]
    for _ in range(warmup):
        oracle.step_worlds(worlds, 1, 0)
    t0 = time.perf_counter()
    total = 0
    for _ in range(steps):
        total += oracle.step_worlds(worlds, 1, 0)
    dt = time.perf_counter() - t0
    nb = sum(s.bubble_count for s in specs)
    return {"value": total / dt if dt > 0 else 0.0, "cores": cores, "steps": steps, "warmup": warmup, "seconds": dt,
            "bubble_substeps": total, "worlds": len(specs), "bubbles": nb}


def cpu_sample_text(leg: dict) -> str:
    return (f"all {leg['worlds']} worlds ({leg['bubbles']} bubbles) of the batched workload, seed 3, {leg['warmup']} "
            f"warm-up + {leg['steps']} timed steps ({leg['seconds']:.1f} s); the reference is Swift + Metal (no "
            f"toolchain, no Metal on this box) so its algorithm runs as the C++ oracle port")


def load_peak():
    try:
        peaks = json.loads(PEAKS_FILE.read_text())
        return float(peaks["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def run_reference(args, rank):
    if rank != 0:
        return 0
    from bubblephysics_gb300 import scenes
    specs = scenes.batched_worlds(args.worlds, seed=3)
    leg = cpu_leg(specs, args.steps, args.warmup)
    value = leg["value"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": leg["seconds"] * 1000.0 / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args, leg["bubbles"]),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": leg["cores"], "kind": "port",
                             "sample": cpu_sample_text(leg)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args, bubbles: int) -> dict:
    """The `config` object both arms print: the same workload name and sizes."""
    return {"workload": f"batched worlds ({args.worlds} worlds per GPU, N~LogUniform[16,1024], r~U[6,24], "
                        f"0-32 bodies, dt=1/60, seed 3)", "worlds": args.worlds, "bubbles": bubbles,
            "l2": "inputs larger than L2: every step touches the state of all worlds (>129 MB)"}


def single_world_rate(spec, ctx, steps: int, warmup: int, contours: bool = False, stop_on_failure: bool = False) -> dict:
    """One world stepped through bp_world_step: device time per step (CUDA events on the library's stream) and
    bubble-substeps per second over `steps` timed steps after `warmup` untimed ones. With stop_on_failure the timed
    steps end at the first step that does not succeed (that step is not counted)."""
    from bubblephysics_gb300.solver import World
    world = World(spec, ctx)
    status, _ = world.step(warmup) if warmup else (0, None)
    statuses, ms, subs = [status], [], 0
    for _ in range(steps):
        status, reps = world.step(1)
        statuses.append(status)
        if stop_on_failure and status != 0:
            break
        ms.append(float(reps["gpu_ms"][0]))
        subs += int(reps["substep_count"][0]) * spec.bubble_count
    keys = world.rigid_keys().size
    contour = None
    if contours:
        # draw-only contours of the published state (bp_world_contours): device time of the contour kernel
        world.contours()
        _, counts, _, _, cms = world.contours()
        contour = {"ms": cms, "samples": int(counts.sum()), "samples_per_s": float(counts.sum()) / (cms / 1e3)}
    world.close()
    total_s = sum(ms) / 1000.0
    done = len(ms)
    return {"bubbles": spec.bubble_count, "segments": len(spec.segments), "bodies": len(spec.bodies),
            "steps": done, "warmup": warmup, "ms_per_step": total_s * 1000.0 / max(done, 1),
            "substeps_per_step": subs / max(spec.bubble_count * done, 1),
            "value": subs / total_s if total_s > 0 else 0.0, "unit": UNIT, "statuses": sorted(set(statuses)),
            "rigid_tree_leaves": keys, "contours": contour}


def single_worlds(ctx, steps: int, large_steps: int, rigid_steps: int) -> dict:
    """The single-world workloads beside the batched headline: the plain world (256 bubbles in 375 x 700, its 60 steps
    from the initial state), the large plain world (65,536 bubbles in 8192^2, grid rebuilt almost every substep;
    whole-GPU team) and the rigid world (16,384 bubbles, ~4,000 static / kinematic bodies in 4096^2, rigid candidates
    through the LBVH, and the same world by brute force for comparison)."""
    import dataclasses
    from bubblephysics_gb300 import _native as N
    from bubblephysics_gb300 import scenes
    out = {"plain_world": single_world_rate(scenes.plain_world(seed=1), ctx, 60, 0)}
    out["large_world"] = single_world_rate(scenes.large_world(), ctx, steps, 3, contours=True)
    # the large world's run from its initial state: the pile needs more substeps every step and reaches the frame limit
    # of 1,024 substeps (BP_E_SUBSTEP_LIMIT) long before 600 steps; the run stops at the first failed step
    full = single_world_rate(scenes.large_world(), ctx, large_steps, 0, stop_on_failure=True)
    full["requested_steps"] = large_steps
    out["large_world_from_start"] = full
    rigid = scenes.rigid_world()
    out["rigid_world"] = single_world_rate(rigid, ctx, rigid_steps, 3)
    brute = dataclasses.replace(rigid, flags=rigid.flags | N.WORLD_NO_RIGID_TREE)
    out["rigid_world_brute_force"] = single_world_rate(brute, ctx, steps, 3)
    t, b = out["rigid_world"]["ms_per_step"], out["rigid_world_brute_force"]["ms_per_step"]
    out["rigid_world"]["speedup_vs_brute_force"] = b / t if t > 0 else None
    return out


def rigid_solver(steps: int = 50, warmup: int = 5, cpu_steps: int = 5) -> dict:
    """The rigid solver on two workloads: jointed chains of box links (every joint kind; 8 x 32, 64 x 32 and
    256 x 32 links), whose bodies meet no other body, stepped by predict + the joint rounds + finish; and a pile of
    256 boxes, circles and capsules dropped on static floors, stepped by the reference's whole rigid step (body-pair
    rows, CCD, 8 rounds of contacts + joints + wall guard). Device time per step and per pass by CUDA events on the
    launching stream (the default stream, torch's current one); the oracle's time per step on one host core."""
    import torch
    from bubblephysics_gb300 import scenes
    from bubblephysics_gb300.rigid import ITERATIONS, RigidSolver
    from oracle.oracle import OracleRigid

    def timed(fn, reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    out = {}
    for chains, links in ((8, 32), (64, 32), (256, 32)):
        scene = scenes.jointed_chains(seed=6, chains=chains, links=links)
        arrays = scene.joint_arrays()
        solver = RigidSolver(scene.bodies, scene.vertices, scene.segments, arrays)
        for _ in range(warmup):
            solver.step_without_contacts(scene.dt, scene.region)
        torch.cuda.synchronize()
        step_ms = timed(lambda: solver.step_without_contacts(scene.dt, scene.region), steps)
        passes = {"predict_ms": timed(lambda: solver.predict(scene.dt), steps),
                  "joint_rounds_ms": timed(lambda: solver.solve_joints(scene.dt, ITERATIONS, ITERATIONS), steps),
                  "finish_ms": timed(lambda: solver.finish(scene.region), steps)}
        oracle = OracleRigid(scene.bodies, scene.vertices, scene.segments, arrays)
        t0 = time.perf_counter()
        for _ in range(cpu_steps):
            oracle.step_without_contacts(scene.dt, scene.region)
        cpu_ms = (time.perf_counter() - t0) * 1000.0 / cpu_steps
        out[f"chains_{chains}x{links}"] = {
            "bodies": len(scene.bodies), "joints": len(arrays.records), "segments": len(scene.segments),
            "rounds": ITERATIONS, "ms_per_step": step_ms, "passes": passes, "safety": solver.safety(),
            "launches_per_step": 4 if len(arrays.records) <= 512 else 3 + 2 * ITERATIONS,
            "cpu_oracle_ms_per_step": cpu_ms, "cpu_cores": 1, "speedup_vs_cpu_oracle": cpu_ms / step_ms,
            "note": "a step = the walls clear (a memset) + predict + the joint rounds + finish"}
    scene = scenes.rigid_pile()
    arrays = scene.joint_arrays()
    solver = RigidSolver(scene.bodies, scene.vertices, scene.segments, arrays, triangles=scene.triangles, row_width=32)
    oracle = OracleRigid(scene.bodies, scene.vertices, scene.segments, arrays, triangles=scene.triangles, row_width=32)
    for _ in range(warmup):
        solver.step(scene.dt, scene.region)
        oracle.step(scene.dt, scene.region)
    torch.cuda.synchronize()
    step_ms = timed(lambda: solver.step(scene.dt, scene.region), steps)
    t0 = time.perf_counter()
    for _ in range(cpu_steps):
        oracle.step(scene.dt, scene.region)
    cpu_ms = (time.perf_counter() - t0) * 1000.0 / cpu_steps
    rows, counts = solver.candidates()
    out["pile_256"] = {
        "bodies": len(scene.bodies), "joints": len(arrays.records), "row_width": 32,
        "row_entries": int(counts[:, 0].sum()), "ms_per_step": step_ms, "safety": solver.safety(),
        "launches_per_step": 5 + 4 * ITERATIONS + 1, "cpu_oracle_ms_per_step": cpu_ms, "cpu_cores": 1,
        "speedup_vs_cpu_oracle": cpu_ms / step_ms,
        "note": "the reference's whole rigid step, after 5 warm-up steps (the pile falling onto the floors)"}
    return out


def plain_world_accuracy(ctx, checkpoints=(1, 10, 30, 60)) -> dict:
    """Part of the CPU-baseline leg: the plain 256-bubble world stepped on the GPU (FP32) against the oracle's FP64 rerun
    of the same steps (the checker). Largest |dx| and |dv| / largest |v| at each checkpoint, and whether the GPU state
    equals the oracle's FP32 run bit for bit there. The world is a dense pile, so FP32 and FP64 separate over time
    (chaotic contact order), while the FP32 runs stay identical."""
    from oracle import oracle
    from bubblephysics_gb300 import scenes
    from bubblephysics_gb300.solver import World
    spec = scenes.plain_world(seed=1)
    gpu, f32, f64 = World(spec, ctx), oracle.OracleWorld(spec, 32), oracle.OracleWorld(spec, 64)
    out, done = [], 0
    for c in checkpoints:
        gpu.step(c - done)
        f32.step(c - done)
        f64.step(c - done)
        done = c
        g, a = gpu.bubbles(), f32.bubbles()
        ref = f64.state64()
        pos = g["center"].astype(np.float64)
        vel = g["velocity"].astype(np.float64)
        vmax = max(float(np.abs(ref[:, 2:4]).max()), 1e-30)
        out.append({"step": c, "max_abs_dx": float(np.abs(pos - ref[:, 0:2]).max()),
                    "max_abs_dv_rel": float(np.abs(vel - ref[:, 2:4]).max()) / vmax,
                    "gpu_equals_fp32_oracle": bool(np.array_equal(g["center"], a["center"]) and
                                                   np.array_equal(g["velocity"], a["velocity"]))})
    gpu.close()
    return {"world": "plain world, 256 bubbles, seed 1", "checkpoints": out}


def log(message: str):
    """Progress of the run on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {message}", file=sys.stderr, flush=True)


def percentile(values, q):
    v = sorted(values)
    return v[min(len(v) - 1, max(0, int(math.ceil(q * len(v))) - 1))] if v else None


def serve_stream(server, arrivals, targets) -> dict:
    """Submits request i when its arrival time has passed, runs the loop in between, then drains. Latency of a
    request = its completion time - its scheduled arrival time (submission lag included)."""
    first = None
    comps = []
    t0 = server.clock()
    i, count = 0, len(arrivals)
    while i < count:
        now = server.clock() - t0
        while i < count and arrivals[i] <= now:
            rid = server.submit(int(targets[i]), 1)
            first = rid if first is None else first
            i += 1
        if server.progress(0):
            comps.append(server.poll())
    comps.append(server.drain(wait_us=50))
    t1 = server.clock()
    done = np.concatenate(comps)
    idx = (done["request_id"] - first).astype(np.int64)
    latency = (done["completed_s"] - (t0 + arrivals[idx])) * 1000.0
    return {"latency_ms": latency, "wall_s": t1 - t0, "statuses": sorted(set(done["status"].tolist()))}


def serving(ctx, args) -> dict:
    """The serving stream: a pool of worlds (N ~ LogUniform[16,4096], batched-world distributions) admitted under a
    120 GB device budget; requests of one step for uniformly random worlds arrive as a Poisson stream. Every world is
    stepped once before the timed stream so the pool starts resident. Measured twice: batched continuous serving and
    the plain per-world path (one launch per world step); plus the saturated throughput of each (all requests at
    once)."""
    from bubblephysics_gb300 import scenes
    from bubblephysics_gb300.solver import Server
    log("serving: generating worlds")
    worlds = scenes.serving_worlds(args.serve_worlds, seed=5, processes=min(os.cpu_count() or 1, 16))
    bubbles = np.array([w.bubble_count for w in worlds], np.int64)
    rng = np.random.default_rng(11)
    arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, args.serve_requests))
    targets = rng.integers(0, len(worlds), args.serve_requests)
    out = {"workload": f"{len(worlds)} resident worlds, N~LogUniform[16,4096], {args.serve_requests} one-step "
                       f"requests, Poisson arrivals at {args.serve_rate:.0f}/s, uniform world choice, 120 GB budget",
           "worlds": len(worlds), "bubbles": int(bubbles.sum()), "requests": args.serve_requests,
           "arrival_rate_per_s": args.serve_rate}
    for mode in ("batched", "per_world"):
        log(f"serving: {mode} pool")
        server = Server(len(worlds), ctx, hbm_budget_bytes=120 << 30, per_world=(mode == "per_world"))
        for spec in worlds:
            server.add_world(spec)
        for w in range(len(worlds)):
            server.submit(w, 1)
        warm = server.drain()
        st0 = server.stats()
        log(f"serving: {mode} stream")
        stream = serve_stream(server, arrivals, targets)
        st1 = server.stats()
        lat = stream["latency_ms"].tolist()
        subs = st1["bubble_substeps"] - st0["bubble_substeps"]
        # saturated: every request of the stream at once
        t0 = server.clock()
        for w in targets:
            server.submit(int(w), 1)
        server.drain(wait_us=50)
        t1 = server.clock()
        st2 = server.stats()
        sat = (st2["bubble_substeps"] - st1["bubble_substeps"]) / (t1 - t0)
        out[mode] = {"latency_ms": {"p50": percentile(lat, 0.50), "p99": percentile(lat, 0.99), "max": max(lat)},
                     "stream_bubble_substeps_per_s": subs / stream["wall_s"], "stream_wall_s": stream["wall_s"],
                     "saturated_bubble_substeps_per_s": sat, "saturated_wall_s": t1 - t0,
                     "requests_per_s_saturated": len(targets) / (t1 - t0),
                     "batches": st1["batches"] - st0["batches"],
                     "mean_worlds_per_batch": (st1["batched_worlds"] - st0["batched_worlds"]) /
                                              max(st1["batches"] - st0["batches"], 1),
                     "resident_worlds": st1["resident"], "resident_gb": st1["resident_bytes"] / 1e9,
                     "evictions": st2["evictions"], "statuses": stream["statuses"],
                     "warmup_statuses": sorted(set(warm["status"].tolist()))}
        server.close()
    # the same stream over the first 4,096 worlds of the pool (the resident-world count of the latency target)
    log("serving: 4096-world pool")
    server = Server(4096, ctx, hbm_budget_bytes=120 << 30)
    for spec in worlds[:4096]:
        server.add_world(spec)
    for w in range(4096):
        server.submit(w, 1)
    server.drain()
    small = serve_stream(server, arrivals, targets % 4096)
    lat = small["latency_ms"].tolist()
    out["batched_4096_worlds"] = {"latency_ms": {"p50": percentile(lat, 0.50), "p99": percentile(lat, 0.99),
                                                 "max": max(lat)}, "statuses": small["statuses"]}
    server.close()
    b, p = out["batched"], out["per_world"]
    out["saturated_speedup_batched_vs_per_world"] = (b["saturated_bubble_substeps_per_s"] /
                                                     p["saturated_bubble_substeps_per_s"])
    return out


def combine_ranks(device_s: float, bubble_substeps: float, dist=None) -> tuple[float, float]:
    """Whole-job timing over ranks: the slowest rank's device time and the sum of all ranks' bubble-substeps."""
    if dist is None:
        return device_s, bubble_substeps
    import torch
    t = torch.tensor([device_s, float(bubble_substeps)], dtype=torch.float64)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(sm[1])


def run_ours(args, rank, world_size, local_rank):
    from bubblephysics_gb300 import scenes
    from bubblephysics_gb300.solver import Batch, Context

    dist = None
    if world_size > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("gloo")

    ctx = Context(local_rank)
    specs = scenes.batched_worlds(args.worlds, seed=3 + rank)
    total_bubbles = sum(s.bubble_count for s in specs)
    batch = Batch(specs, ctx, use_graph=True, autotune=not args.no_autotune)
    sampler = ClockSampler(local_rank)
    sampler.start()
    st, _ = batch.step(args.warmup)
    _, subs0, launches0 = batch.counters()
    if dist:
        dist.barrier()
    step_ms, statuses = [], []
    rebuild_bubbles = 0
    timed0 = time.time()
    for _ in range(args.steps):
        status, reps = batch.step(1)  # returns after the step's stream synchronisation
        statuses.append(status)
        step_ms.append(float(reps["gpu_ms"][0]))
        rebuild_bubbles += int((reps["rebuild_count"].astype(np.int64) * batch.sizes).sum())
    timed1 = time.time()
    _, subs1, launches1 = batch.counters()
    device_s = sum(step_ms) / 1000.0
    bubble_substeps = subs1 - subs0
    degree_sum = batch.adjacency_entries()
    mean_degree = degree_sum / max(total_bubbles, 1)
    builds = total_bubbles * args.steps + rebuild_bubbles
    alg_bytes = algorithmic_bytes(bubble_substeps, builds, mean_degree)
    kernel_launches = (launches1 - launches0)
    # step kernels, plus the report accumulation and the on-device scheduler of every step (one CUDA graph per step)
    gpu_launches = kernel_launches + 2 * args.steps
    device_s_all, substeps_all = combine_ranks(device_s, float(bubble_substeps), dist)
    value = substeps_all / device_s_all if device_s_all > 0 else 0.0

    # end to end through the C ABI with host buffers
    host, keep = pinned_buffer(total_bubbles)
    batch.read_state(host)
    _, e2e_s0, _ = batch.counters()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        batch.write_state(host)
        batch.step(1)
        batch.read_state(host)
    e2e_wall = time.perf_counter() - t0
    clocks = sampler.stop(timed=(timed0, timed1))
    _, e2e_s1, _ = batch.counters()
    e2e_value = (e2e_s1 - e2e_s0) / e2e_wall if e2e_wall > 0 else 0.0

    # the plain per-world launch path on the same worlds, from the same initial state
    per_world = None
    if args.per_world_steps > 0:
        plain = Batch(specs, ctx, per_world_launch=True, use_graph=False)
        plain.step(1)
        _, p0, pl0 = plain.counters()
        _, preps = plain.step(args.per_world_steps)
        _, p1, pl1 = plain.counters()
        pms = float(preps["gpu_ms"][0])
        fused = Batch(specs, ctx, use_graph=True)
        fused.step(1)
        _, f0, _ = fused.counters()
        _, freps = fused.step(args.per_world_steps)
        _, f1, _ = fused.counters()
        fms = float(freps["gpu_ms"][0])
        launches = (pl1 - pl0) // args.per_world_steps
        per_world = {"value": (p1 - p0) / (pms / 1000.0), "unit": UNIT, "launches_per_step": launches,
                     "ms_per_step": pms / args.per_world_steps,
                     "device_ms_per_launch": pms / args.per_world_steps / max(launches, 1),
                     "note": "one launch per world, one world per block (a warp for worlds of <= 64 bubbles), "
                             "launches back to back on one stream; device_ms_per_launch is the mean device time of a "
                             "launch, i.e. of one world's step with one team",
                     "batched_same_steps": (f1 - f0) / (fms / 1000.0),
                     "speedup_batched_vs_per_world": ((f1 - f0) / fms) / ((p1 - p0) / pms) if pms > 0 and p1 > p0 else None,
                     "steps": args.per_world_steps}
        plain.close()
        fused.close()

    if rank != 0:
        if dist:
            dist.barrier()
        return 0

    # single-world and serving measurements are one-GPU figures: they run in one-process runs only
    singles = (single_worlds(ctx, args.single_steps, args.large_steps, args.rigid_steps)
               if args.single_steps > 0 and world_size == 1 else None)
    served = serving(ctx, args) if args.serve_requests > 0 and world_size == 1 else None
    peak, peak_kind = load_peak()
    achieved = alg_bytes / device_s / 1e9 if device_s > 0 else 0.0
    traffic = None
    try:
        prof = json.loads(PROFILE_FILE.read_text())
        # dram bytes per bubble-substep measured by ncu on a smaller batch, scaled to one launch of this workload
        per_unit = float(prof["dram_bytes_per_bubble_substep"])
        traffic = per_unit * bubble_substeps / max(kernel_launches, 1)
    except Exception:
        traffic = None
    alg_per_launch = alg_bytes / max(kernel_launches, 1)
    # the CPU baseline: the reference arm's measurement itself, run as the reference arm runs (a fresh process: this
    # one holds the CUDA context, torch and the GPU work's threads, which slowed the oracle's OpenMP team by 2x)
    cpu_steps = args.steps if args.cpu_steps <= 0 else min(args.cpu_steps, args.steps)
    ref = subprocess.run([sys.executable, str(Path(__file__).resolve()), "--impl", "reference", "--steps", str(cpu_steps),
                          "--warmup", str(args.warmup), "--worlds", str(args.worlds)], capture_output=True, text=True)
    ref_line = json.loads(ref.stdout.strip().splitlines()[-1])
    leg = {"value": ref_line["value"], "cores": ref_line["cpu_baseline"]["cores"],
           "sample": ref_line["cpu_baseline"]["sample"]}
    accuracy = plain_world_accuracy(ctx) if world_size == 1 else None
    rigid = None
    if world_size == 1 and args.single_steps > 0:
        try:
            rigid = rigid_solver()
        except Exception as exc:  # the headline line is printed whatever happens to this side measurement
            rigid = {"error": f"{type(exc).__name__}: {exc}"}
    lat = sorted(step_ms)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": device_s_all * 1000.0 / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(args, total_bubbles),
                       substeps_per_step_mean=bubble_substeps / max(total_bubbles * args.steps, 1),
                       mean_adjacency_degree=mean_degree, statuses=sorted(set(statuses))),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": total_bubbles * 16,
                "d2h_bytes_per_step": total_bubbles * 16, "steps": args.e2e_steps,
                "note": "C ABI bp_batch_write_state + bp_batch_step + bp_batch_read_state from pinned host memory, wall clock"},
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)],
                       "max": lat[-1],
                       "note": "device time of one step of all worlds together; the per-request step latency of the "
                               "serving loop is serving.*.latency_ms"},
        "per_world_launch": per_world,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "persistent_step_kernel", "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg_per_launch,
                     "bytes_model": "76 + 40*k per bubble-substep, 96 + 8*k per bubble grid build (k = mean degree)"},
        "cpu_baseline": {"value": leg["value"], "unit": UNIT, "cores": leg["cores"], "kind": "port",
                         "sample": leg["sample"] + " (bench.py --impl reference, run as a separate process)"},
        "accuracy_fp32_vs_fp64": accuracy,
        "clocks": clocks,
        "gpu_launches": gpu_launches,
        "single_worlds": singles,
        "serving": served,
        "rigid_solver": rigid,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


def run_case(name: str) -> int:
    """One small launch of a chosen kernel for profilers (ncu -k ... python bench.py --case NAME); prints its status.
      batch     persistent_step_kernel, schedule_kernel, accumulate_kernel: 4 steps of the 4,096-world batch, autotuned
      batch512  the same with a fixed schedule (512-thread blocks, worlds of <= 64 bubbles in 64-thread groups)
      large     large_step_kernel: 3 steps of the 65,536-bubble world
      rigid     large_step_kernel: 3 steps of the 16,384-bubble rigid world (3,017 bodies, 5,652 edges, LBVH)
      served    served_step_kernel: 3 rounds of one-step requests over 512 resident worlds
      contour   contour_kernel: contours of the 65,536-bubble world after 3 steps
      hit       hit_test_kernel: 65,536 query points on the 256-bubble world
      sensor    sensor_overlap_kernel, sensor_compact_kernel: 64 circle sensors on the 256-bubble world
      events    contact_events_kernel: contact events of the 256-bubble world, 3 steps
      noalloc   noalloc_step_kernel: 3 allocation-free steps of the 256-bubble world
      state     write_state_kernel, read_state_kernel, sum_kernel: the end-to-end state copies of the 4,096-world batch
                (903 k bubbles) and its adjacency-entry count, 3 times each
      chains    rigid_predict_kernel, rigid_joint_round_kernel, rigid_apply_round_kernel, rigid_finish_kernel: 3 steps
                of 256 x 32 jointed links without body contacts
      pile      every rigid kernel: 3 whole rigid steps of 256 boxes, circles and capsules dropped on static floors"""
    import ctypes as C
    from bubblephysics_gb300 import _native as N
    from bubblephysics_gb300 import scenes
    from bubblephysics_gb300.solver import Batch, Context, Server, World
    ctx = Context(0)
    if name in ("chains", "pile"):
        from bubblephysics_gb300.rigid import RigidSolver
        if name == "chains":
            scene = scenes.jointed_chains(seed=6, chains=256, links=32)
            solver = RigidSolver(scene.bodies, scene.vertices, scene.segments, scene.joint_arrays())
            step = solver.step_without_contacts
        else:
            scene = scenes.rigid_pile()
            solver = RigidSolver(scene.bodies, scene.vertices, scene.segments, scene.joint_arrays(),
                                 triangles=scene.triangles, row_width=32)
            step = solver.step
        for _ in range(3):
            step(scene.dt, scene.region)
        print("bodies", len(scene.bodies), "safety", solver.safety())
        return 0 if solver.safety() == 0 else 1
    if name in ("batch", "batch512"):
        kw = dict(autotune=True) if name == "batch" else dict(threads_per_world=512, warp_world_max=64, group_width=64)
        b = Batch(scenes.batched_worlds(4096, seed=3), ctx, use_graph=True, **kw)
        st, r = b.step(4)
        print("status", st, "ms per step", float(r["gpu_ms"][0]) / 4, b.tuning())
        return 0 if st == N.OK else 1
    if name == "state":
        b = Batch(scenes.batched_worlds(4096, seed=3), ctx, use_graph=True, threads_per_world=512, warp_world_max=64,
                  group_width=64)
        host, keep = pinned_buffer(int(b.sizes.sum()))
        b.read_state(host)
        for _ in range(3):
            b.write_state(host)
            b.read_state(host)
            entries = b.adjacency_entries()
        print("bubbles", int(b.sizes.sum()), "adjacency entries", entries)
        return 0
    if name in ("large", "rigid"):
        st, r = World(scenes.large_world() if name == "large" else scenes.rigid_world(), ctx).step(3)
        print("status", st, "substeps", r["substep_count"].tolist())
        return 0 if st == N.OK else 1
    if name == "served":
        worlds = scenes.serving_worlds(512, seed=5)
        server = Server(len(worlds), ctx)
        for spec in worlds:
            server.add_world(spec)
        statuses = set()
        for _ in range(3):
            for w in range(len(worlds)):
                server.submit(w, 1)
            statuses |= set(server.drain()["status"].tolist())
        print("statuses", sorted(statuses))
        return 0 if statuses == {N.OK} else 1
    spec = scenes.large_world() if name == "contour" else scenes.plain_world(seed=1)
    world = World(spec, ctx)
    if name == "sensor":
        sensors = []
        for q in range(64):
            s = N.Sensor()
            s.id = 10_000 + q
            s.position[:] = [float(20 + (q % 8) * 45), float(40 + (q // 8) * 80)]
            s.radius = 30.0
            s.flags = N.SENSOR_ENTER_EVENTS | N.SENSOR_EXIT_EVENTS
            sensors.append(s)
        world.set_sensors(sensors)
    st, _ = world.step(3)
    if name == "contour":
        print("contour ms", world.contours()[-1])
    elif name == "hit":
        points = np.random.default_rng(1).uniform([0, 0], [375, 700], (65536, 2)).astype(np.float32)
        print("hits", int(world.hit_test(points)[2].sum()))
    elif name == "sensor":
        print("sensor events", len(world.sensor_events()))
    elif name == "events":
        ids = set(int(i) for i in spec.bubbles["id"])
        for _ in range(3):
            world.step(1)
            print("events", world.contact_events(ids).size)
    elif name == "noalloc":
        import torch
        spec.candidate_limit = 32
        bubbles = torch.from_numpy(spec.bubbles.view(np.uint8).copy()).cuda()
        segments = torch.from_numpy(np.ascontiguousarray(spec.segments).view(np.uint8).copy()).cuda()
        reports = torch.zeros(3 * 96, dtype=torch.uint8, device="cuda")
        st = N.library().bp_world_step_noalloc(C.byref(spec.desc()), C.c_void_p(bubbles.data_ptr()),
                                               spec.bubble_count, C.c_void_p(segments.data_ptr()),
                                               len(spec.segments), 3, C.c_void_p(reports.data_ptr()), None)
        torch.cuda.synchronize()
    else:
        raise SystemExit(f"unknown case {name}")
    print("status", st)
    return 0 if st == N.OK else 1


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--worlds", type=int, default=4096)
    p.add_argument("--e2e-steps", type=int, default=10)
    p.add_argument("--per-world-steps", type=int, default=2)
    p.add_argument("--cpu-steps", type=int, default=0,
                   help="timed steps of the CPU baseline leg (0: the same as --steps, the reference arm's sample)")
    p.add_argument("--single-steps", type=int, default=10,
                   help="timed steps of the rigid world by brute force (0: skip the single worlds)")
    p.add_argument("--large-steps", type=int, default=600, help="timed steps of the 65,536-bubble large world")
    p.add_argument("--rigid-steps", type=int, default=300, help="timed steps of the rigid world")
    p.add_argument("--serve-worlds", type=int, default=8192)
    p.add_argument("--serve-requests", type=int, default=20000, help="requests of the serving stream (0: skip)")
    p.add_argument("--serve-rate", type=float, default=50000.0, help="Poisson arrival rate of the serving stream")
    p.add_argument("--no-autotune", action="store_true", help="keep the default schedule (profiling runs)")
    p.add_argument("--case", default=None, help="run one small case of one kernel for a profiler (see run_case)")
    args = p.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.case:
        return run_case(args.case)
    rank = env_int("RANK", 0)
    world_size = env_int("WORLD_SIZE", 1)
    local_rank = env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        return run_reference(args, rank)
    return run_ours(args, rank, world_size, local_rank)


if __name__ == "__main__":
    sys.exit(main())
