"""Benchmark of the GB300 lattice time step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload precision512|default128|plain64|profile256|batch64|profile_batch64|serve|serve_light|precision_study]

Metric: cell-updates/s (one cell-update = one full SSP-RK3 step of one
cell), on the 512^3 precision-study workload by default: periodic 512^3
lattice, 256 seeded bubbles nucleated at t = 0 (radius 1.15 R_c), eta drawn
log-uniform in [0.02, 1.0] from the seed, FP32 state with FP64 reductions and
FP64 con2prim where gamma > 3.  A step is one SSP-RK3 step of the whole
lattice (three fused stage launches).  The lattice (9.7 GB) is far larger
than L2, so no flush is needed between steps.

`value` is device-timed with CUDA events on the library's stream, the state
resident in HBM.  `e2e` is a headless-style solve through the C ABI: the
initial state is uploaded from pinned host memory, K steps advance with a
diagnostics readback every 10 steps, and the final state is copied back to
pinned host memory, all inside the timed region.

`--impl reference` times the CPU restatement of the reference's algorithm
(the oracle's native build; the reference itself is Rust/WGSL and cannot
run here) on all host cores, each step one SSP-RK3 step of the z < 32 slab
of the workload's lattice as nucleated at t = 0 -- the same sample the GPU
arm's cpu_baseline leg times.

With --gpus N > 1 (under torchrun) every rank advances its own replica of
the workload (the lattices are independent; no data-path collective):
`value` is the sum over ranks, timed by the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "bubble-simulation_gb300"))

BYTES_PER_CELL_UPDATE = 192  # compulsory FP32 traffic of the three stages: 48 + 72 + 72


def workload(name: str) -> dict:
    rng = np.random.default_rng(20251203)
    if name == "precision512":
        eta = float(math.exp(rng.uniform(math.log(0.02), math.log(1.0))))
        return dict(name="512^3 periodic, 256 bubbles at t=0 (1.15 R_c), eta log-uniform[0.02,1] "
                         f"draw {eta:.4f}, FP32 state + FP64 reductions + FP64 con2prim where gamma>3",
                    grid=(512, 512, 512), bubbles=256, nucleation="simultaneous", duration=1.0,
                    eta=eta, precision="mixed", seed=1)
    if name == "default128":
        return dict(name="128^3 periodic, 12 bubbles, nucleation times uniform over the first 200 steps, "
                         "eta 0.3, FP32", grid=(128, 128, 128), bubbles=12, nucleation="uniform",
                    duration=40.0, eta=0.3, precision="single", seed=1)
    if name == "profile256":
        return dict(name="256^3 periodic, 32 bubbles at t=0 (1.15 R_c), eta 0.3, FP32 state + FP64 "
                         "reductions + FP64 con2prim where gamma>3 (small case of precision512 for ncu)",
                    grid=(256, 256, 256), bubbles=32, nucleation="simultaneous", duration=1.0, eta=0.3,
                    precision="mixed", seed=1)
    if name == "plain64":
        return dict(name="64^3 periodic, 1 bubble at the centre (1.15 R_c), eta 0.3, FP32",
                    grid=(64, 64, 64), bubbles=1, nucleation="centre", duration=1.0, eta=0.3,
                    precision="single", seed=1)
    raise SystemExit(f"unknown workload {name}")


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def ncu_traffic(wl: str) -> float | None:
    """DRAM bytes per cell per stage launch from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "stage_kernel_traffic_256cubed.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_cell_update:"):
            return float(line.split(":")[1])
    return None


def ncu_flops() -> float | None:
    """FP32 operations per cell-update of the stage kernel from the committed
    ncu summary (FADD + FMUL + 2 FFMA, paired forms counted per lane), if any."""
    p = ROOT / "profiles" / "stage_kernel_flops_256cubed.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("fp32_flop_per_cell_update:"):
            return float(line.split(":")[1])
    return None


# Nominal FP32 (CUDA-core) rate of a GB300: 152 SMs x 128 lanes x 2 (FMA) x 2.07 GHz.
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def make_spec(bubble, wl: dict):
    model = bubble.Model(eta=wl["eta"])
    return bubble.SimulationSpec(model=model, grid=wl["grid"], nucleation=wl["nucleation"],
                                 bubbles=wl["bubbles"], nucleation_duration=wl["duration"],
                                 seed=wl["seed"], precision=wl["precision"], math="fast")


def workload_slab(wl: dict, zs: int = 32, warm_steps: int = 2):
    """The CPU baseline's sample of a workload: the z < zs slab of its lattice
    (periodic in z over the slab) as nucleated at t = 0 by the workload's own
    schedule (every bubble, minimum-image distances in the full lattice, the
    reference's tanh profile), then warm_steps SSP-RK3 steps of the oracle.
    Returns the warmed OracleSim on the native timing build.  Built on the
    host alone, so the GPU arm's cpu_baseline leg and the reference arm time
    exactly the same sample."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    oracle.build(native=True)
    nx, ny, nz = wl["grid"]
    zs = min(zs, nz)
    m = dict(oracle.DEFAULT_MODEL, eta=wl["eta"])
    d = oracle.derived(m)
    sched = oracle.make_schedule(wl["nucleation"], wl["bubbles"], d["seed_radius"], wl["grid"], wl["duration"],
                                 wl["seed"])
    phi = np.zeros((zs, ny, nx), dtype=np.float32)
    phi_b, l_w, dx = float(m["phi_b"]), float(d["wall_width"]), float(m["dx"])

    def min_image(a, n):
        return (a + 0.5 * n) % n - 0.5 * n

    for t, pos, r0 in sched:
        if t > 0.0:
            continue
        cut = r0 * dx + 9.5 * l_w  # tanh saturates beyond: the profile is 0
        span = int(math.ceil(cut / dx)) + 1
        xs = np.arange(int(pos[0]) - span, int(pos[0]) + span + 1) % nx
        ys = np.arange(int(pos[1]) - span, int(pos[1]) + span + 1) % ny
        zz = np.arange(zs)
        dzs = min_image(zz - pos[2], nz)
        keep = np.abs(dzs) * dx < cut
        if not keep.any():
            continue
        ddx = min_image(xs - pos[0], nx)[None, None, :]
        ddy = min_image(ys - pos[1], ny)[None, :, None]
        ddz = dzs[keep][:, None, None]
        r = np.sqrt(ddx * ddx + ddy * ddy + ddz * ddz) * dx
        prof = (0.5 * phi_b * (1.0 - np.tanh((r - r0 * dx) / l_w))).astype(np.float32)
        sub = np.ix_(zz[keep], ys, xs)
        phi[sub] = np.maximum(phi[sub], prof)
    sim = oracle.OracleSim((nx, ny, zs), model=m, native=True)
    f, u = sim.state()
    f[:, 0] = phi.reshape(-1)
    sim.set_state(f, u)
    for _ in range(warm_steps):
        sim.record_step()
    return sim


def slab_sample_text(wl: dict, sim, threads: int) -> str:
    import platform

    nx, ny, zs = sim.grid
    flag = "-mcpu=native" if platform.machine() in ("aarch64", "arm64") else "-march=native"
    return (f"SSP-RK3 steps of the z<{zs} slab ({nx}x{ny}x{zs}, periodic) of the {wl['grid'][0]}x"
            f"{wl['grid'][1]}x{wl['grid'][2]} workload nucleated at t=0 by its own schedule "
            f"({wl['bubbles']} bubbles), warmed 2 steps; FP32 oracle (the reference's kernel structure: "
            f"primitives pass, two HLL fluxes per face) built g++ -O3 {flag} -fopenmp, {threads} threads")


def cpu_baseline(wl: dict, seconds_budget: float = 20.0) -> dict:
    """Time the oracle's native build on all host cores over the workload's
    CPU sample (workload_slab), and one step of its first planes on one
    thread."""
    sim = workload_slab(wl)
    nx, ny, zs = sim.grid
    threads = sim.L.oracle_threads()
    t0 = time.perf_counter()
    steps = 0
    while True:
        sim.record_step()
        steps += 1
        if time.perf_counter() - t0 > seconds_budget * 0.5 or steps >= 8:
            break
    dt = time.perf_counter() - t0
    cells = nx * ny * zs
    # one thread: one step of the slab's first 8 planes
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    f, u = sim.state()
    z1 = min(8, zs)
    sim1 = oracle.OracleSim((nx, ny, z1), model=sim.model, native=True)
    sim1.set_state(f.reshape(zs, ny, nx, 2)[:z1].reshape(-1, 2), u.reshape(zs, ny, nx, 4)[:z1].reshape(-1, 4))
    sim.L.oracle_set_threads(1)
    t1 = time.perf_counter()
    sim1.record_step()
    dt1 = time.perf_counter() - t1
    sim.L.oracle_set_threads(threads)
    return {"value": cells * steps / dt, "unit": "cell-updates/s", "cores": threads,
            "kind": "port", "value_1_thread": nx * ny * z1 / dt1, "cpu_model": cpu_model(),
            "nproc": os.cpu_count(), "sample": slab_sample_text(wl, sim, threads) +
            f"; {steps} step(s) timed; value_1_thread: one step of its first {z1} planes on one thread"}


def max_over_ranks(ms: float, dist, device: str) -> float:
    """The whole job's clock: the slowest rank's time (ms).  `dist` is
    torch.distributed (None for one rank); `device` holds the reduced tensor
    ("cuda" under NCCL, "cpu" under gloo)."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_model() -> str:
    """The host CPU's model name (x86 'model name', Arm implementer/part)."""
    try:
        text = open("/proc/cpuinfo").read()
    except OSError:
        return platform.processor() or "unknown"
    for key in ("model name", "Model name"):
        for line in text.splitlines():
            if line.startswith(key):
                return line.split(":", 1)[1].strip()
    impl = [ln.split(":", 1)[1].strip() for ln in text.splitlines() if ln.startswith("CPU implementer")]
    part = [ln.split(":", 1)[1].strip() for ln in text.splitlines() if ln.startswith("CPU part")]
    if impl and part:
        return f"Arm implementer {impl[0]} part {part[0]} ({platform.machine()})"
    return platform.processor() or platform.machine()


def run_reference(args, wl: dict, world: int, rank: int) -> int:
    """The reference arm: its algorithm on the host cores (the oracle's native
    build; the reference itself is Rust/WGSL and cannot run here), on the same
    CPU sample as the GPU arm's cpu_baseline leg (workload_slab)."""
    if rank != 0:
        return 0
    sim = workload_slab(wl)
    nx, ny, zs = sim.grid
    threads = sim.L.oracle_threads()
    for _ in range(max(args.warmup - 2, 0)):
        sim.record_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.record_step()
    dt = time.perf_counter() - t0
    cells = nx * ny * zs
    value = cells * args.steps / dt
    sample = slab_sample_text(wl, sim, threads) + "; one slab step per step"
    line = {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": wl["name"], "grid": list(wl["grid"]), "sample_grid": [nx, ny, zs]},
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                             "sample": sample, "cpu_model": cpu_model()},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def batch_specs(bubble, n: int, seed: int = 20251203):
    """The batched-ensemble workload: n lattices, edges drawn from {32, 48, 64, 96},
    one bubble at the centre, seed factor U[0.7, 1.5], eta log-U[0.02, 1]."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n):
        edge = int(rng.choice([32, 48, 64, 96]))
        model = bubble.Model(eta=float(math.exp(rng.uniform(math.log(0.02), math.log(1.0)))),
                             seed_value=float(rng.uniform(0.7, 1.5)))
        specs.append(bubble.SimulationSpec(model=model, grid=(edge,) * 3, nucleation="centre", bubbles=1,
                                           seed=k + 1, math="fast"))
    return specs


def run_batch_profile(args) -> int:
    """Small case of the batched ensemble for a profiler: the batch64 lattices,
    direct launches (no CUDA graph), no autotuning, a few steps per launch."""
    import torch
    import bubble_gb300 as bubble

    bubble.load()
    specs = batch_specs(bubble, args.lattices)
    cells = sum(s.grid[0] ** 3 for s in specs)
    b = bubble.Batch(specs, autotune=False, use_graph=False)
    b.advance(2)  # nucleation and a first launch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        b.advance(5)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    info = b.info()
    b.close()
    print(json.dumps({"metric": "cell-updates/s", "value": cells * 15 / dt, "unit": "cell-updates/s",
                      "impl": "gb300-batch-profile", "config": {"workload": f"{args.lattices} lattices of the "
                      "batch64 workload, direct launches, no autotuning, 3 launches of 5 steps", "cells": cells},
                      "batch_info": info}), flush=True)
    return 0


def run_batch(args) -> int:
    """Batched ensemble (solves/s): one persistent graph-captured launch per
    chunk of steps for all lattices, against the same plain kernels run one
    lattice at a time (each with its autotuned z chunk)."""
    import torch
    import bubble_gb300 as bubble

    bubble.load()
    n, steps = args.lattices, args.batch_steps
    specs = batch_specs(bubble, n)
    cells = sum(s.grid[0] ** 3 for s in specs)
    t0 = time.perf_counter()
    b = bubble.Batch(specs)
    setup_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    chunk = 100
    done = 0
    while done < steps:
        b.advance(min(chunk, steps - done))
        done += min(chunk, steps - done)
    broken_b = [b.diagnostics(k).broken_fraction for k in range(n)]
    t_batch = time.perf_counter() - t0
    info = b.info()
    b.close()
    lz_cache = {}
    t_plain = 0.0
    broken_p = []
    for s in specs:
        if s.grid not in lz_cache:
            lz_cache[s.grid] = bubble.autotune_chunk(s.grid, 16, "fast")
        sim = bubble.Simulation(s)
        sim.set_tile(16, lz_cache[s.grid])
        sim.synchronize()
        t0 = time.perf_counter()
        sim.advance(steps)
        d = sim.diagnostics()
        t_plain += time.perf_counter() - t0
        broken_p.append(d.broken_fraction)
        sim.close()
    agree = sum((a > 0) == (p > 0) for a, p in zip(broken_b, broken_p))
    line = {"metric": "solves/s", "value": n / t_batch, "unit": "solves/s", "n_gpus": 1, "steps": steps,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic", "impl": "gb300-batch",
            "config": {"workload": f"{n} lattices, edges from {{32,48,64,96}}, 1 bubble, seed factor U[0.7,1.5], "
                                   f"eta log-U[0.02,1], {steps} steps, FP32 fast", "cells": cells},
            "plain_solves_per_s": n / t_plain, "speedup_vs_plain": t_plain / t_batch,
            "batch_cell_updates_per_s": cells * steps / t_batch,
            "plain_cell_updates_per_s": cells * steps / t_plain,
            "outcome_agreement": f"{agree}/{n}", "grown_batch": sum(x > 0 for x in broken_b),
            "batch_info": info, "setup_s": setup_s}
    print(json.dumps(line), flush=True)
    return 0


SERVE_EDGES = {"serve": (48, 64, 128, 192, 256), "serve_light": (48, 64, 96, 128)}


def serve_requests(bubble, n: int, seed: int = 20251203, edges=SERVE_EDGES["serve"]):
    """The serving workload: edges from {48, 64, 128, 192, 256}, 1-32 bubbles
    with nucleation times uniform over the first 200 steps, eta log-U[0.02, 1],
    seed factor U[0.9, 1.5], 500-3000 steps; Poisson arrivals at 20 req/s."""
    rng = np.random.default_rng(seed)
    reqs, t = [], 0.0
    for k in range(n):
        t += float(rng.exponential(1.0 / 20.0))
        edge = int(rng.choice(list(edges)))
        model = bubble.Model(eta=float(math.exp(rng.uniform(math.log(0.02), math.log(1.0)))),
                             seed_value=float(rng.uniform(0.9, 1.5)))
        spec = bubble.SimulationSpec(model=model, grid=(edge,) * 3, nucleation="uniform",
                                     bubbles=int(rng.integers(1, 33)), nucleation_duration=40.0, seed=k + 1,
                                     math="fast")
        reqs.append((t, spec, int(rng.integers(500, 3001))))
    return reqs


def percentile(xs, p):
    xs = sorted(xs)
    pos = p * (len(xs) - 1)
    i = int(math.floor(pos))
    j = min(i + 1, len(xs) - 1)
    return xs[i] + (pos - i) * (xs[j] - xs[i])


def run_serve(args) -> int:
    """Serving stream: requests arrive (Poisson, 20/s) while others run and join
    the batched launch at the next round; latency = completion - arrival.  The
    plain path answers the same requests one at a time in arrival order."""
    import bubble_gb300 as bubble

    bubble.load()
    edges = SERVE_EDGES[args.workload]
    reqs = serve_requests(bubble, args.requests, edges=edges)
    n = len(reqs)

    def serve(policy):
        srv = bubble.Server(math="fast", chunk_steps=50, policy=policy, chunk_planes=args.chunk_planes)
        base = srv.now()
        arrival_of, i, done = {}, 0, []
        while len(done) < n:
            now = srv.now() - base
            while i < n and reqs[i][0] <= now:
                rid = srv.submit(reqs[i][1], reqs[i][2])
                arrival_of[rid] = base + reqs[i][0]
                i += 1
            busy = srv.tick()
            done += srv.poll()
            if not busy and i < n:
                time.sleep(max(0.0, reqs[i][0] - (srv.now() - base)))
        lat = [r["done_s"] - arrival_of[r["id"]] for r in done]
        span = max(r["done_s"] for r in done) - (base + reqs[0][0])
        st = srv.stats()
        srv.close()
        return lat, span, st

    lat, span, st = serve("fifo")
    lat_sj, span_sj, _ = serve("shortest")
    # plain path: one request at a time, in arrival order
    durations = []
    for _, spec, steps in reqs:
        sim = bubble.Simulation(spec)
        sim.synchronize()
        t0 = time.perf_counter()
        sim.advance(steps)
        sim.diagnostics()
        durations.append(time.perf_counter() - t0)
        sim.close()
    free_at, plain_lat, finish = 0.0, [], 0.0
    for (arr, _, _), d in zip(reqs, durations):
        start = max(free_at, arr)
        free_at = start + d
        plain_lat.append(free_at - arr)
        finish = free_at
    cells = sum(s.grid[0] ** 3 * k for _, s, k in reqs)
    # The bound on any schedule of these requests: every cell-update at the
    # fastest rate the plain path reaches on any one of them (its largest
    # lattices fill the GPU alone); the plain path's busy time over that.
    work = [s.grid[0] ** 3 * k for _, s, k in reqs]
    rates = [w / d for w, d in zip(work, durations)]
    r_max = max(rates)
    per_edge = {}
    for (_, s, _), r in zip(reqs, rates):
        per_edge.setdefault(s.grid[0], []).append(r)
    bound = {"fastest_plain_rate": r_max, "ratio_bound": sum(durations) / (sum(work) / r_max),
             "plain_rate_by_edge": {str(e): sum(v) / len(v) for e, v in sorted(per_edge.items())}}
    edge_txt = ",".join(str(e) for e in edges)
    line = {"metric": "solves/s", "value": n / span, "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic", "impl": "gb300-serve",
            "config": {"workload": f"{n} requests, Poisson 20/s, edges from {{{edge_txt}}}, 1-32 bubbles, "
                                   "eta log-U[0.02,1], seed factor U[0.9,1.5], 500-3000 steps, FP32 fast"},
            "speedup_vs_plain": (n / span) / (n / (finish - reqs[0][0])), "bound": bound,
            "p50_latency_s": percentile(lat, 0.5), "p99_latency_s": percentile(lat, 0.99),
            "cell_updates_per_s": cells / span, "policy": "fifo with backfill, 24 M resident cells", "chunk_planes": args.chunk_planes or 64,
            "shortest_first": {"solves_per_s": n / span_sj, "p50_latency_s": percentile(lat_sj, 0.5),
                               "p99_latency_s": percentile(lat_sj, 0.99)},
            "plain": {"solves_per_s": n / (finish - reqs[0][0]), "p50_latency_s": percentile(plain_lat, 0.5),
                      "p99_latency_s": percentile(plain_lat, 0.99), "cell_updates_per_s": cells / sum(durations)},
            "server_stats": st}
    print(json.dumps(line), flush=True)
    return 0


def run_precision_study(args) -> int:
    """The precision-study configuration against the FP64 CUDA oracle: the same
    seeded lattice (edge --study-grid, the 512^3 config's bubble density, eta
    drawn as in precision512) advanced --study-steps steps in FP64 (DOUBLE),
    FP32 MIXED and the FP32 perturbation form.  Every 100 steps the total
    energy (FP64 sums); drift = E / E0 - 1 with E0 the first report after
    every bubble is in (src/headless.rs:69-75); at the end, per-field max
    error of each FP32 form against FP64, relative to the field's FP64 max."""
    import numpy as np
    import torch
    import bubble_gb300 as bubble

    bubble.load()
    n, steps = args.study_grid, args.study_steps
    wl = workload("precision512")
    bubbles = max(1, round(256 * (n / 512) ** 3))
    model = bubble.Model(eta=wl["eta"])
    out, states = {}, {}
    for prec in ("double", "mixed", "perturbation"):
        spec = bubble.SimulationSpec(model=model, grid=(n, n, n), nucleation="simultaneous", bubbles=bubbles,
                                     nucleation_duration=1.0, seed=wl["seed"], precision=prec, math="fast")
        series, e0 = [], None
        t0 = time.perf_counter()
        with bubble.Simulation(spec) as sim:
            done = 0
            while done < steps:
                k = min(100, steps - done)
                sim.advance(k)
                done += k
                d = sim.diagnostics()
                if e0 is None and sim.remaining_bubbles() == 0:
                    e0 = d.mean_energy_f64
                series.append({"step": done, "mean_energy_f64": d.mean_energy_f64,
                               "drift": (d.mean_energy_f64 / e0 - 1.0) if e0 else None,
                               "broken": d.broken_fraction, "max_v": d.max_velocity})
            f, u = sim.copy_state()
        torch.cuda.synchronize()
        if prec == "perturbation":
            u = u.astype(np.float64)
            u[:, 0] += float(bubble.derived(model)["e_ref"])
        states[prec] = (f.astype(np.float64), u.astype(np.float64))
        out[prec] = {"seconds": time.perf_counter() - t0, "series": series}
    f64, u64 = states["double"]
    names = ("phi", "pi", "E", "Zx", "Zy", "Zz")
    for prec in ("mixed", "perturbation"):
        f, u = states[prec]
        err = {}
        for c, nm in enumerate(names):
            a = f[:, c] if c < 2 else u[:, c - 2]
            b = f64[:, c] if c < 2 else u64[:, c - 2]
            err[nm] = float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
        e = u64[:, 0] - float(bubble.derived(model)["e_ref"])
        err["E - e_ref"] = float(np.abs((u[:, 0] - float(bubble.derived(model)["e_ref"])) - e).max()
                                 / max(np.abs(e).max(), 1e-300))
        out[prec]["field_err_vs_fp64"] = err
        d32 = out[prec]["series"][-1]["drift"]
        d64 = out["double"]["series"][-1]["drift"]
        out[prec]["final_drift"] = d32
        out[prec]["drift_minus_fp64_drift"] = d32 - d64
    line = {"metric": "energy drift and per-field error vs the FP64 CUDA oracle", "impl": "gb300-precision-study",
            "config": {"workload": f"{n}^3 periodic, {bubbles} bubbles at t=0 (1.15 R_c), eta {wl['eta']:.4f}, "
                                   f"{steps} steps, fast arithmetic", "grid": [n, n, n]},
            "final_drift_fp64": out["double"]["series"][-1]["drift"], "forms": out}
    print(json.dumps(line), flush=True)
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="precision512")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--lattices", type=int, default=64, help="batch64 workload: number of lattices")
    ap.add_argument("--batch-steps", type=int, default=1000, help="batch64 workload: steps per solve")
    ap.add_argument("--chunk-planes", type=int, default=0,
                    help="serve workload: z planes per work item of a lattice (0: the server's default)")
    ap.add_argument("--requests", type=int, default=24, help="serve workload: number of requests")
    ap.add_argument("--study-grid", type=int, default=256, help="precision_study workload: lattice edge")
    ap.add_argument("--study-steps", type=int, default=3000, help="precision_study workload: steps")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.workload == "profile_batch64":
        return run_batch_profile(args)
    if args.workload == "batch64":
        return run_batch(args)
    if args.workload in SERVE_EDGES:
        return run_serve(args)
    if args.workload == "precision_study":
        return run_precision_study(args)
    wl = workload(args.workload)
    world, rank, local = dist_setup()

    if args.impl == "reference":
        return run_reference(args, wl, world, rank)

    import torch

    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist

    import bubble_gb300 as bubble

    bubble.load()
    stream = torch.cuda.Stream()
    sim = bubble.Simulation(make_spec(bubble, wl))
    sim.set_stream(stream.cuda_stream)
    cells = sim.cell_count()
    # warm-up: nucleation at t = 0 plus W steps
    sim.advance(args.warmup)
    sim.synchronize()
    ty, lz = sim.tile()

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    # the e2e leg below replays these same K steps from this state
    state0 = None if args.no_e2e else sim.copy_state()
    launches0 = sim.launches()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    with ClockSampler(local) as clocks:
        with torch.cuda.stream(stream):
            start.record(stream)
            sim.advance(args.steps)
            end.record(stream)
        end.synchronize()
    barrier()
    launches = sim.launches() - launches0
    ms = max_over_ranks(start.elapsed_time(end), pg, "cuda")
    ms_per_step = ms / args.steps
    value = world * cells * args.steps / (ms * 1e-3)

    # e2e through the C ABI: pinned host state in, K steps, report every 10,
    # state out; the state is the one the timed region started from, so both
    # legs advance the same steps of the same evolution
    e2e = None
    if not args.no_e2e:
        field, fluid = state0
        pin_f = torch.from_numpy(field).pin_memory()
        pin_u = torch.from_numpy(fluid).pin_memory()
        out_f = torch.empty_like(pin_f).pin_memory()
        out_u = torch.empty_like(pin_u).pin_memory()
        L = bubble.load()
        state_bytes = field.nbytes + fluid.nbytes
        # untimed pass over the same buffers (first DMA use of fresh pinned
        # pages), which also gives the box's pinned copy rates
        c0 = time.perf_counter()
        bubble._lib.check(L.bubble_load_state(sim.handle, pin_f.data_ptr(), pin_u.data_ptr()))
        c1 = time.perf_counter()
        bubble._lib.check(L.bubble_copy_state(sim.handle, out_f.data_ptr(), out_u.data_ptr()))
        c2 = time.perf_counter()
        barrier()

        def e2e_leg():
            t0 = time.perf_counter()
            bubble._lib.check(L.bubble_load_state(sim.handle, pin_f.data_ptr(), pin_u.data_ptr()))
            t1 = time.perf_counter()
            done = reports = 0
            while done < args.steps:
                n = min(10, args.steps - done)
                sim.advance(n)
                sim.diagnostics()
                reports += 1
                done += n
            t2 = time.perf_counter()
            bubble._lib.check(L.bubble_copy_state(sim.handle, out_f.data_ptr(), out_u.data_ptr()))
            t3 = time.perf_counter()
            return reports, {"upload": (t1 - t0) * 1e3, "steps_and_reports": (t2 - t1) * 1e3,
                             "download": (t3 - t2) * 1e3, "total": (t3 - t0) * 1e3}

        # three legs, each from the same start state; the median leg is reported
        with ClockSampler(local) as e2e_clocks:
            legs = [e2e_leg() for _ in range(3)]
        reports = legs[0][0]
        totals = sorted(leg[1]["total"] for leg in legs)
        med = next(leg[1] for leg in legs if leg[1]["total"] == totals[1])
        e2e_ms = max_over_ranks(totals[1], pg, "cuda")
        e2e_val = world * cells * args.steps / (e2e_ms * 1e-3)
        e2e = {"value": e2e_val, "unit": "cell-updates/s",
               "h2d_bytes_per_step": state_bytes / args.steps,
               "d2h_bytes_per_step": (state_bytes + reports * 88) / args.steps,
               "pinned_copy_gbs": {"h2d": state_bytes / (c1 - c0) / 1e9, "d2h": state_bytes / (c2 - c1) / 1e9},
               "legs_ms": [round(t, 2) for t in totals], "median_leg_ms": {k: round(v, 2) for k, v in med.items()},
               "clocks": e2e_clocks.summary(),
               "what": "pinned host state (the timed region's start) -> the same K steps with diagnostics "
                       "every 10 -> pinned host state; median of three legs"}

    peak, peak_kind = peaks()
    achieved = BYTES_PER_CELL_UPDATE * cells / (ms_per_step * 1e-3) / 1e9
    traffic_per_cell = ncu_traffic(args.workload)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": (traffic_per_cell * cells / 3) if traffic_per_cell else None,
                "algorithmic_bytes_per_launch": BYTES_PER_CELL_UPDATE * cells / 3,
                "kernel": "stage_kernel (3 launches per step)"}
    flop_per_cell = ncu_flops()
    fp32 = None
    if flop_per_cell:
        tf = flop_per_cell * cells / (ms_per_step * 1e-3) / 1e12
        fp32 = {"achieved": tf, "unit": "TFLOP/s", "flop_per_cell_update": flop_per_cell,
                "nominal_peak": FP32_NOMINAL_TFLOPS, "frac_of_nominal": tf / FP32_NOMINAL_TFLOPS}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl)

    if rank == 0:
        line = {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": wl["name"], "grid": list(wl["grid"]), "cells": cells,
                           "tile": [16 if ty == 16 else 32, ty, lz], "l2": "inputs larger than L2 (no flush)",
                           "parallelism": f"replicas x{world}" if world > 1 else "single lattice"},
                "roofline": roofline, "fp32": fp32, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches, "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)
    sim.close()
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
