"""Generate the committed golden fixtures from the oracle and the reference's docs.

    python tests/golden/make_golden.py --reference DIR [--skip-128]

Writes into tests/golden/:
  published_numerics.json  the reference's published single-bubble and
                           quiescent tables (its docs/NUMERICS.md) and the
                           grow/collapse threshold table (its docs/PHYSICS.md)
  single_bubble_128.json   the oracle's diagnostics of that published case
                           (128^3, 1 bubble, simultaneous, seed 1) at step 100,
                           beside the published row
  cases.npz                small per-cell cases: initial state, oracle state
                           after N steps (FP32 and FP64), and the parameters

The reference tree is read only here, at generation time; tests read the
JSON/NPZ files.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "oracle"))
import oracle  # noqa: E402


def parse_tables(numerics_md: Path) -> dict:
    text = numerics_md.read_text()
    out = {"single_bubble": {}, "quiescent": {}}
    # Single bubble table: step time broken R_eq max|v| K E/E0
    sb = re.search(r"### Single bubble, default parameters.*?```(.*?)```", text, re.S)
    for line in sb.group(1).strip().splitlines()[1:]:
        p = line.split()
        out["single_bubble"][p[0]] = dict(time=float(p[1]), broken_pct=float(p[2].rstrip("%")),
                                          r_eq=float(p[3]), max_v=float(p[4]), k=float(p[5]),
                                          e_ratio=float(p[6]))
    q = re.search(r"### Quiescent state is exactly preserved.*?```(.*?)```", text, re.S)
    for line in q.group(1).strip().splitlines()[1:]:
        p = line.split()
        out["quiescent"][p[0]] = dict(broken_pct=float(p[1].rstrip("%")), max_v=float(p[2]), k=float(p[3]))
    return out


def parse_threshold(physics_md: Path) -> dict:
    """The grow/collapse table of docs/PHYSICS.md: broken % after 700 steps."""
    text = physics_md.read_text()
    t = {}
    for line in text.splitlines():
        m = re.match(r"\|\s*(0\.\d+)\s*\|\s*[\d.]+\s*\|\s*[\d.]+\s*\|(.*)\|\s*$", line)
        if not m:
            continue
        cells = [c.strip() for c in m.group(2).split("|")]
        if len(cells) != 4:
            continue
        for sf, c in zip(("0.90", "0.96", "1.00", "1.15"), cells):
            t[f"{m.group(1)}_{sf}"] = None if c == "collapsed" else float(c.rstrip("%"))
    return t


def perturbed_state(sim: "oracle.OracleSim", seed: int, amp: float) -> None:
    """Add a smooth seeded velocity field and pressure bumps to the current slot."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = sim.grid
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    fluid = sim.fluid[sim.cur].reshape(nz, ny, nx, 4).astype(np.float64)
    e = fluid[..., 0]
    for c in (1, 2, 3):
        kx, ky, kz = rng.integers(1, 3, size=3)
        ph = rng.uniform(0, 2 * np.pi)
        fluid[..., c] += amp * e * np.sin(2 * np.pi * (kx * x / nx + ky * y / ny + kz * z / nz) + ph)
    fluid[..., 0] *= 1.0 + 0.3 * amp * np.cos(2 * np.pi * (x / nx + 2 * y / ny)) ** 2
    # a sharp jump so the limiter and HLL see a shock
    fluid[nz // 2:, :, : nx // 3, 0] *= 1.5
    sim.fluid[sim.cur] = fluid.reshape(-1, 4).astype(sim.dtype)


def relativistic_state(sim: "oracle.OracleSim", seed: int, v_peak: float = 0.995) -> int:
    """Add a smooth relativistic blob to the current slot: inside a seeded ball
    of radius R (a third of the shortest axis) the fluid moves along a seeded
    direction at |v| = v_peak up to R/2 and v_peak cos^2 beyond, reaching 0
    at R, at 1 to 1.5 times the background pressure, so the ball holds cells
    at every Lorentz factor from 1 to 1/sqrt(1 - v_peak^2) (gamma > 3 where
    |v| > 0.943).  Conserved variables
    are built in FP64 from (v, p) (bag model: w = 4p, E = w W^2 - p,
    Z = w W^2 v) and rounded once.  Returns the number of cells whose FP32
    recovery gives v^2 > 8/9."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = sim.grid
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    c = rng.uniform(0.3, 0.7, size=3) * np.array([nx, ny, nz])
    rad = max(min(nx, ny, nz) / 3.0, 4.0)
    d = [np.minimum(np.abs(a - ca), n - np.abs(a - ca)) for a, ca, n in ((x, c[0], nx), (y, c[1], ny), (z, c[2], nz))]
    r = np.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2)
    inside = r < rad
    ramp = np.cos(np.pi * np.clip(r / rad - 0.5, 0.0, 0.5)) ** 2
    speed = np.where(inside, v_peak * ramp, 0.0)
    n = rng.normal(size=3)
    n /= np.linalg.norm(n)
    e_ref = float(sim.d["e_ref"])
    p = e_ref / 3.0 * (1.0 + 0.5 * np.where(inside, ramp, 0.0))
    w2 = 1.0 / (1.0 - speed ** 2)
    ww = 4.0 * p * w2
    fluid = sim.fluid[sim.cur].reshape(nz, ny, nx, 4).astype(np.float64)
    sel = inside
    fluid[..., 0] = np.where(sel, ww - p - (e_ref if sim.pert else 0.0), fluid[..., 0])
    for k in range(3):
        fluid[..., 1 + k] = np.where(sel, ww * speed * n[k], fluid[..., 1 + k])
    sim.fluid[sim.cur] = fluid.reshape(-1, 4).astype(sim.dtype)
    # cells the FP32 recovery puts above gamma = 3
    u = sim.fluid[sim.cur].astype(np.float64)
    e = np.maximum(u[:, 0] + (e_ref if sim.pert else 0.0), 1e-30)
    z2 = (u[:, 1:] ** 2).sum(axis=1)
    pp = (e * e - z2) / (e + np.sqrt(np.maximum(4 * e * e - 3 * z2, 0)))
    v2 = z2 / (e + pp) ** 2
    return int((v2 > 8.0 / 9.0).sum())


CASES = [
    # name, grid, bubbles (centre mode, radius), steps, velocity amplitude, seed
    ("odd", (9, 11, 13), 3.5, 12, 0.30, 1),
    ("tile_partial", (40, 20, 18), 6.0, 10, 0.20, 2),
    ("flat", (64, 8, 8), 5.0, 8, 0.45, 3),
]


def make_cases() -> dict:
    arrays = {}
    for name, grid, r, steps, amp, seed in CASES:
        for prec in ("f32", "f64"):
            sched = oracle.make_schedule("centre", 1, r, grid, 10.0, 1)
            sim = oracle.OracleSim(grid, schedule=sched, precision=prec)
            sim.record_nucleation()
            perturbed_state(sim, seed, amp)
            f0, u0 = sim.state()
            sim.advance(steps)
            f1, u1 = sim.state()
            arrays[f"{name}_{prec}_field0"] = f0
            arrays[f"{name}_{prec}_fluid0"] = u0
            arrays[f"{name}_{prec}_field"] = f1
            arrays[f"{name}_{prec}_fluid"] = u1
        arrays[f"{name}_grid"] = np.array(grid)
        arrays[f"{name}_steps"] = np.array(steps)
    return arrays


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("BUBBLE_REFERENCE"),
                    help="the reference source tree (default: $BUBBLE_REFERENCE)")
    ap.add_argument("--skip-128", action="store_true")
    a = ap.parse_args()
    if not a.reference:
        ap.error("--reference (or BUBBLE_REFERENCE) must name the reference source tree")
    oracle.build()
    pub = parse_tables(Path(a.reference) / "docs" / "NUMERICS.md")
    pub["threshold_700"] = parse_threshold(Path(a.reference) / "docs" / "PHYSICS.md")
    (HERE / "published_numerics.json").write_text(json.dumps(pub, indent=1))
    np.savez_compressed(HERE / "cases.npz", **make_cases())
    if not a.skip_128:
        grid = (128, 128, 128)
        d = oracle.derived(oracle.DEFAULT_MODEL)
        sched = oracle.make_schedule("simultaneous", 1, d["seed_radius"], grid, 60.0, 1)
        sim = oracle.OracleSim(grid, schedule=sched)
        t0 = time.time()
        sim.advance(100)
        diag = sim.diagnostics()
        out = {"case": "128^3, 1 bubble, simultaneous, seed 1, eta 0.3, cfl 0.2 (FP32 oracle)",
               "seconds": time.time() - t0, "threads": oracle.lib().oracle_threads(),
               "schedule": [[float(e[0]), [float(p) for p in e[1]], float(e[2])] for e in sched],
               "oracle_step_100": {k: float(v) for k, v in diag.items()},
               "published": pub["single_bubble"]}
        (HERE / "single_bubble_128.json").write_text(json.dumps(out, indent=1))
        print(json.dumps(out["oracle_step_100"], indent=1), out["seconds"])
    return 0


if __name__ == "__main__":
    sys.exit(main())
