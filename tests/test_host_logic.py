"""Host logic of the library through its C ABI, on the CPU.

The product's derived constants and nucleation schedules are compared bit
for bit with the oracle's independent restatements; the reference's own
host unit tests (cited) are restated against the library.
"""
from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import PKG, ROOT

f32 = np.float32

MODELS = [
    dict(),
    dict(eps_ratio=0.15, lambda_=0.1),
    dict(eps_ratio=0.6, lambda_=1.5, alpha=0.02, eta=0.02),
    dict(eps_ratio=0.95, cfl=0.5, seed_value=0.7),
    dict(seed_kind="cells", seed_value=7.5),
]


def as_model(bubble, d):
    return bubble.Model(**d)


@pytest.mark.parametrize("m", MODELS)
def test_derived_matches_oracle_bit_for_bit(bubble, oracle_mod, m):
    prod = bubble.derived(as_model(bubble, m))
    ref = oracle_mod.derived(dict(oracle_mod.DEFAULT_MODEL, **m))
    for k, v in ref.items():
        assert f32(prod[k]).tobytes() == f32(v).tobytes(), (k, prod[k], v)


@pytest.mark.parametrize("mode", ["simultaneous", "exponential", "centre", "uniform"])
@pytest.mark.parametrize("count,grid,seed", [(12, (64, 64, 64), 7), (1, (128, 128, 128), 1),
                                             (40, (96, 64, 80), 12345), (256, (512, 512, 512), 3)])
def test_schedule_matches_oracle_bit_for_bit(bubble, oracle_mod, mode, count, grid, seed):
    radius = 15.333334
    prod = bubble.make_schedule(mode, count, radius, grid, 60.0, seed)
    ref = oracle_mod.make_schedule(mode, count, radius, grid, 60.0, seed)
    assert len(prod) == len(ref) == count
    for (t, p, r), (tr, pr, rr) in zip(prod, ref):
        assert f32(t).tobytes() == f32(tr).tobytes()
        assert f32(r).tobytes() == f32(rr).tobytes()
        for a, b in zip(p, pr):
            assert f32(a).tobytes() == f32(b).tobytes()


def test_pcg_stream_matches_oracle(oracle_mod):
    # the oracle's pure-Python Pcg64Mcg against a direct big-integer statement
    g = oracle_mod.Pcg64Mcg.seed_from_u64(1)
    mult = 0x2360ED051FC65DA44385DF649FCCF645
    st = g.state
    for _ in range(5):
        st = (st * mult) % (1 << 128)
        rot = st >> 122
        x = ((st >> 64) ^ st) & ((1 << 64) - 1)
        want = ((x >> rot) | (x << (64 - rot))) & ((1 << 64) - 1) if rot else x
        assert g.next_u64() == want


# src/physics.rs:387-401 through the library
def test_schedule_ordering_and_bounds(bubble):
    ev = bubble.make_schedule("exponential", 12, 8.0, (64, 64, 64), 40.0, 7)
    assert len(ev) == 12
    assert all(a[0] <= b[0] for a, b in zip(ev, ev[1:]))
    for t, pos, _ in ev:
        assert 0.0 <= t <= 40.0 + 1e-3
        assert all(0.0 <= p <= 64.0 for p in pos)


# src/physics.rs:191-217 messages
@pytest.mark.parametrize("m,msg", [
    (dict(eps_ratio=0.0), "eps_ratio must lie in (0, 1)"),
    (dict(eps_ratio=1.0), "eps_ratio must lie in (0, 1)"),
    (dict(lambda_=0.0), "lambda must be positive"),
    (dict(alpha=-1.0), "alpha must be positive"),
    (dict(eta=-0.1), "eta must be non-negative"),
    (dict(cfl=0.6), "cfl must lie in (0, 0.5]; see docs/NUMERICS.md"),
    (dict(seed_value=0.0), "seed factor must be positive"),
    (dict(seed_kind="cells", seed_value=-1.0), "seed radius must be positive"),
])
def test_validate_messages(bubble, oracle_mod, m, msg):
    assert bubble.validate_model(as_model(bubble, m)) == msg
    assert oracle_mod.validate(dict(oracle_mod.DEFAULT_MODEL, **m)) == msg


def test_sub_critical_seed_is_valid(bubble):
    assert bubble.validate_model(bubble.Model(seed_value=0.5)) is None


# src/gpu/sim.rs:1057-1068
def test_stage_slots(bubble, oracle_mod):
    for cur in range(3):
        assert bubble.stage_slots(cur) == oracle_mod.stage_slots(cur)


# src/gpu/sim.rs:1108-1116
def test_rk3_third_stage_weights_do_not_sum_to_one_in_binary32(bubble):
    """The origin of the FP32 scheme's systematic drift: the reference's third
    stage weights fl(1/3) + fl(2/3) sum to exactly 1 + 2^-25 in binary32 (the
    other stages' weights are exact), so over evolving cells a0 U^n + a1 U1
    comes out 2.98e-8 too large on average (round to nearest of a biased
    value).  The fast kernels evaluate U^n + a1 (U1 - U^n), unbiased."""
    (a0, a1), (b0, b1), (c0, c1) = [tuple(map(np.float32, p)) for p in bubble.rk3_coefficients()]
    assert float(a0) + float(a1) == 1.0 and float(b0) + float(b1) == 1.0
    assert float(c0) + float(c1) == 1.0 + 2.0 ** -25
    rng = np.random.default_rng(0)
    un = rng.uniform(0.12, 0.13, 200_000).astype(np.float32)
    u1 = (un * (1.0 + rng.normal(0.0, 1e-4, un.size))).astype(np.float32)
    exact = un.astype(np.float64) / 3.0 + u1.astype(np.float64) * (2.0 / 3.0)
    biased = (c0 * un).astype(np.float32) + (c1 * u1).astype(np.float32)
    unbiased = un + (c1 * (u1 - un)).astype(np.float32)
    rel_b = np.mean(biased.astype(np.float64) / exact - 1.0)
    rel_u = np.mean(unbiased.astype(np.float64) / exact - 1.0)
    assert abs(rel_b - 2.0 ** -25) < 0.2 * 2.0 ** -25, rel_b
    assert abs(rel_u) < 0.05 * 2.0 ** -25, rel_u


def test_rk3(bubble, oracle_mod):
    for (a0, a1), (b0, b1) in zip(bubble.rk3_coefficients(), oracle_mod.RK3_F32):
        assert f32(a0) == b0 and f32(a1) == b1
        assert abs(a0 + a1 - 1.0) < 1e-6 and a0 >= 0 and a1 > 0


# src/gpu/sim.rs:1080-1083, for this layout: 3 slots x 24 B, no prim cache,
# no visualisation texture
def test_lattice_bytes(bubble):
    assert bubble.lattice_bytes((100, 10, 10)) == 10_000 * 72


# src/gpu/sim.rs:1085-1106 with the 72 B/cell memory model
def test_max_cubic_size(bubble):
    side, lim = bubble.max_cubic_size(2_147_483_648, 1 << 60)
    assert not lim and side == int((2_147_483_648 // 16) ** (1 / 3) + 1e-9)
    tight, lim2 = bubble.max_cubic_size(2_147_483_648, 1_000_000_000)
    assert lim2 and tight < side
    assert bubble.lattice_bytes((tight,) * 3) <= 1_000_000_000
    assert bubble.max_cubic_size(2_147_483_648, None)[0] == side
    assert bubble.max_cubic_size(1024, 1024)[0] == 8
    # beyond the reference's 2048-cell axis cap: the 32-bit cell index
    assert bubble.max_cubic_size(1 << 62, None)[0] == 1625


# src/gpu/vram.rs:162-207
def test_vram_budget(bubble):
    assert bubble.vram_available(24_000_000_000, 23_000_000_000, 3_000_000_000) == 20_000_000_000
    assert bubble.vram_available(8_000_000_000) == 8_000_000_000
    assert bubble.lattice_budget(1_000_000_000, 10_000_000_000) > 9_000_000_000
    assert bubble.lattice_budget(1_000, 0) == 850
    assert bubble.vram_available(8_000_000_000, 7_000_000_000, 7_500_000_000) == 0


def test_exports_every_declared_symbol(bubble):
    L = bubble.load()
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(bubble_\w+)\s*\(", text)
    names = sorted(set(names))
    assert len(names) > 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    declared = {s[0] for s in bubble._lib.SIGNATURES}
    assert set(names) <= declared | {"bubble_sim"}, set(names) - declared


def test_no_device_means_loud_failure(bubble):
    """Without a GPU, creating a simulation fails with a CUDA error, never a CPU path."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(bubble.BubbleError) as e:
        bubble.Simulation(bubble.SimulationSpec(grid=(16, 16, 16)))
    assert e.value.code == bubble._lib.ERR_CUDA


def test_lattice_above_32_bit_cell_index_is_rejected(bubble):
    """The stage kernels index cells in 32 bits: a lattice of 2^32 cells or
    more is refused before any device work (2048 x 2048 x 1024 is exactly
    2^32), while the axis limit alone would accept it."""
    with pytest.raises(bubble.BubbleError) as e:
        bubble.Simulation(bubble.SimulationSpec(grid=(2048, 2048, 1024)))
    assert e.value.code == bubble._lib.ERR_INVALID
    assert "4294967296 cells" in str(e.value)


# ---- CLI (src/config.rs:209-242, src/main.rs) -------------------------------
CLI = PKG / "lib" / "bubble-sim"


def run_cli(*args):
    return subprocess.run([str(CLI), *args], capture_output=True, text=True, timeout=60)


def test_cli_rejects_bad_grid(bubble):
    r = run_cli("--grid", "1,2", "--headless", "1")
    assert r.returncode != 0 and "not a lattice size" in r.stderr
    r = run_cli("--grid", "abc", "--headless", "1")
    assert r.returncode != 0


def test_cli_rejects_small_grid(bubble):
    r = run_cli("--grid", "4", "--headless", "1")
    assert r.returncode == 1 and "needs at least 8 cells" in r.stderr


def test_cli_rejects_unresolvable_wall(bubble):
    r = run_cli("--lambda", "50", "--headless", "1")
    assert r.returncode == 1 and "cells thick" in r.stderr


def test_cli_rejects_bad_model(bubble):
    r = run_cli("--cfl", "0.7", "--headless", "1")
    assert r.returncode == 1 and "cfl must lie in (0, 0.5]" in r.stderr
    r = run_cli("--bubbles", "0", "--headless", "1")
    assert r.returncode == 1 and "--bubbles must be at least 1" in r.stderr


def test_cli_help(bubble):
    r = run_cli("--help")
    assert r.returncode == 0 and "--headless" in r.stdout
