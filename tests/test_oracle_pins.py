"""Pin the CPU oracle against the reference's own known-answer tests.

Each test restates an assertion of the reference's unit tests (cited) or a
number the reference publishes, and checks the oracle (oracle/oracle.py +
oracle/oracle.cpp) against it.  No GPU is involved.
"""
from __future__ import annotations

import json
import math

import numpy as np
import pytest

from conftest import GOLDEN

f32 = np.float32


def v_of(d, lam):
    def v(p):
        p = f32(p)
        return f32(f32(f32(f32(0.5) * d["m2"]) * f32(p * p)) - f32(f32(d["delta"] * f32(p * p * p)) / f32(3.0))
                   + f32(f32(0.25) * lam) * f32(p ** 4))

    def dv(p):
        p = f32(p)
        return f32(p * f32(f32(d["m2"] - f32(d["delta"] * p)) + f32(f32(lam * p) * p)))

    return v, dv


# src/physics.rs:316-336 potential_has_the_requested_shape
def test_potential_has_the_requested_shape(oracle_mod):
    m = dict(oracle_mod.DEFAULT_MODEL)
    d = oracle_mod.derived(m)
    lam = f32(m["lambda_"])
    v, dv = v_of(d, lam)
    assert d["m2"] > 0.0
    assert abs(dv(1.0)) < 1e-6
    assert abs(v(1.0) + d["eps"]) < 1e-6
    top = max(v(i / 100.0) for i in range(100))
    assert top > 0.0


# src/physics.rs:338-344 degenerate_limit_is_the_symmetric_double_well
def test_degenerate_limit(oracle_mod):
    m = dict(oracle_mod.DEFAULT_MODEL, eps_ratio=1e-6)
    d = oracle_mod.derived(m)
    assert abs(d["m2"] - 0.5 * 0.5) < 1e-4
    assert abs(d["delta"] - 1.5 * 0.5) < 1e-4


# src/physics.rs:348-362 critical_radius_is_never_smaller_than_the_wall
@pytest.mark.parametrize("eps_ratio", [0.05, 0.2, 0.3, 0.6, 0.95])
@pytest.mark.parametrize("lam", [0.1, 0.5, 1.5])
def test_critical_to_wall_ratio(oracle_mod, eps_ratio, lam):
    d = oracle_mod.derived(dict(oracle_mod.DEFAULT_MODEL, eps_ratio=eps_ratio, lambda_=lam))
    ratio = d["critical_radius"] / d["wall_width"]
    assert abs(ratio - d["critical_to_wall_ratio"]) < 1e-3 * ratio
    assert ratio > 1.0


# src/physics.rs:364-385
def test_seed_radius_modes(oracle_mod):
    base = dict(oracle_mod.DEFAULT_MODEL, seed_kind="critical", seed_value=1.15)
    d = oracle_mod.derived(base)
    assert abs(d["seed_radius"] - 1.15 * d["critical_radius"]) < 1e-4
    softer = oracle_mod.derived(dict(base, eps_ratio=0.6))
    assert softer["seed_radius"] < d["seed_radius"]
    fixed = dict(oracle_mod.DEFAULT_MODEL, seed_kind="cells", seed_value=7.5)
    assert abs(oracle_mod.derived(fixed)["seed_radius"] - 7.5) < 1e-6
    assert abs(oracle_mod.derived(dict(fixed, eps_ratio=0.6))["seed_radius"] - 7.5) < 1e-6
    sub = dict(oracle_mod.DEFAULT_MODEL, seed_value=0.5)
    assert oracle_mod.validate(sub) is None
    assert oracle_mod.derived(sub)["seed_radius"] < oracle_mod.derived(sub)["critical_radius"]


# src/physics.rs:387-401 schedule_respects_ordering_and_bounds
def test_schedule_ordering_and_bounds(oracle_mod):
    ev = oracle_mod.make_schedule("exponential", 12, 8.0, (64, 64, 64), 40.0, 7)
    assert len(ev) == 12
    for a, b in zip(ev, ev[1:]):
        assert a[0] <= b[0]
    for t, pos, _ in ev:
        assert 0.0 <= t <= 40.0 + 1e-3
        for p in pos:
            assert 0.0 <= p <= 64.0


def test_schedule_min_separation(oracle_mod):
    r = 8.0
    ev = oracle_mod.make_schedule("simultaneous", 6, r, (128, 128, 128), 10.0, 3)
    n = [f32(128)] * 3
    for i in range(len(ev)):
        for j in range(i):
            assert oracle_mod.periodic_distance(ev[i][1], ev[j][1], n) > 2.5 * r


# src/gpu/sim.rs:1057-1068 stage_slots_never_alias_output_with_input
def test_stage_slots(oracle_mod):
    for cur in range(3):
        slots = oracle_mod.stage_slots(cur)
        for i, o in slots:
            assert i != o and o != cur
        assert slots[2][1] == (cur + 1) % 3


# src/gpu/sim.rs:1108-1116 rk3_coefficients_are_consistent
def test_rk3_convex(oracle_mod):
    for a0, a1 in oracle_mod.RK3_F32:
        assert abs(float(a0) + float(a1) - 1.0) < 1e-6
        assert a0 >= 0.0 and a1 > 0.0


# src/gpu/sim.rs:1070-1078 parameter_blocks_have_the_expected_size
def test_sim_params_size(oracle_mod):
    assert oracle_mod.lib().oracle_params_size_f32() == 96
    m = oracle_mod.DEFAULT_MODEL
    assert oracle_mod._sim_params(np.float32, m, (8, 8, 8)).nbytes == 96
    assert oracle_mod._sim_params(np.float64, m, (8, 8, 8)).nbytes == oracle_mod.lib().oracle_params_size_f64()


def test_fp64_oracle_tracks_fp32_oracle(oracle_mod):
    """The two instances solve the same problem: they differ by rounding only."""
    grid = (20, 16, 12)
    sched = oracle_mod.make_schedule("centre", 1, 5.0, grid, 1.0, 1)
    out = []
    for prec in ("f32", "f64"):
        sim = oracle_mod.OracleSim(grid, schedule=sched, precision=prec)
        sim.advance(30)
        out.append(sim.state())
    for a, b in zip(out[0], out[1]):
        scale = np.max(np.abs(b), axis=0)
        assert np.max(np.max(np.abs(a - b), axis=0) / scale) < 1e-4
    assert np.max(np.abs(out[1][0][:, 0])) > 0.3  # the (collapsing) bubble is still there


def test_oracle_tanh_is_accurate(oracle_mod):
    L = oracle_mod.lib()
    xs = np.concatenate([np.linspace(-25, 25, 4001), np.geomspace(1e-12, 0.6, 200)])
    for x in xs:
        t = L.oracle_tanh_f64(float(x))
        ref = math.tanh(float(x))
        assert abs(t - ref) <= 1e-15 * max(abs(ref), 1e-300), (x, t, ref)
    # the FP32 tanh of the FP32 profile: within 4 ulp of the exact value, and
    # exactly +-1 where a correctly rounded tanhf is
    rng = np.random.default_rng(0)
    xs = np.concatenate([np.linspace(-14, 14, 20001), rng.uniform(-10, 10, 20000),
                         np.geomspace(1e-30, 1.0, 400), -np.geomspace(1e-30, 1.0, 400)]).astype(np.float32)
    worst = 0.0
    for x in xs:
        t = np.float32(L.oracle_tanh_f32(float(x)))
        ref = math.tanh(float(x))
        ulp = float(np.spacing(np.float32(abs(ref)))) if ref != 0.0 else 1e-45
        err = abs(float(t) - ref) / ulp
        worst = max(worst, err)
        assert err <= 4.0, (x, t, ref, err)
        if abs(float(x)) > 9.5:
            assert abs(float(t)) == 1.0
    assert worst > 0.0


# docs/NUMERICS.md:163-175: the quiescent state is a discrete fixed point
def test_quiescent_state_is_exact(oracle_mod):
    sim = oracle_mod.OracleSim((12, 10, 9))
    f0, u0 = sim.state()
    sim.advance(20)
    f1, u1 = sim.state()
    assert np.array_equal(f0, f1) and np.array_equal(u0, u1)
    d = sim.diagnostics()
    assert d["max_velocity"] == 0.0 and d["broken_fraction"] == 0.0


def test_energy_drift_stays_at_discretisation_level(oracle_mod):
    # A sub-critical bubble (6 cells against R_c = 13.3) collapsing in a 24^3
    # box: the sharpest dynamics a small lattice offers.  Total energy is
    # conserved by the continuum equations; the drift is discretisation error.
    grid = (24, 24, 24)
    d = oracle_mod.derived(oracle_mod.DEFAULT_MODEL)
    sched = oracle_mod.make_schedule("centre", 1, 6.0, grid, 10.0, 1)
    sim = oracle_mod.OracleSim(grid, schedule=sched)
    sim.advance(1)
    e0 = sim.diagnostics()["mean_energy_f64"]
    sim.advance(80)
    dd = sim.diagnostics()
    assert abs(dd["mean_energy_f64"] / e0 - 1.0) < 1e-3
    assert dd["broken_fraction"] == 0.0  # the sub-critical bubble is gone
    assert d["dt"] == f32(0.2)


def test_oracle_single_bubble_fixture_is_consistent():
    """The committed 128^3 oracle run (tests/golden/make_golden.py) of the
    reference's documented single-bubble command: schedule, seed radius and
    a growing bubble.  The GPU tests compare the CUDA path with it."""
    g = json.loads((GOLDEN / "single_bubble_128.json").read_text())
    (t, pos, r), = g["schedule"]
    assert t == 0.0 and abs(r - 15.333334) < 1e-5
    row = g["oracle_step_100"]
    r_eq = (row["broken_fraction"] * 128 ** 3 * 3 / (4 * math.pi)) ** (1 / 3)
    assert r_eq > r  # supercritical seed grows
    assert 0.0 < row["max_velocity"] < 1.0 and row["sum_energy"] > 0.0
