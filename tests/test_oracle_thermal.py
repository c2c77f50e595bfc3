"""The oracle's thermal potential (include/bubble.h BUBBLE_EOS_THERMAL,
docs/EOS.md:120-150) on the CPU.

The reference has no implementation of this recipe, so these tests pin the
restatement by the properties the recipe names: the inversion recovers
(v, p) of states built in FP64 from (T, phi, v); gamma = A = 0 is the bag
model to rounding; the quiescent state is a fixed point; a uniform broken
phase hotter than T_ref feels the restoring force -gamma (T^2 - T_ref^2)
phi of the thermal mass term; and total energy, with the field's V(phi, 0),
is conserved as well as the bag model conserves it (the recipe's step 4:
the diagnostic measures the energy the solver conserves).
"""
from __future__ import annotations

import numpy as np
import pytest


def bounds(oracle_mod):
    a = float(oracle_mod.derived(oracle_mod.DEFAULT_MODEL)["a_rad"])
    return a, a / 6.0, a / np.sqrt(2.0)  # a, gamma_max, A_max at T_ref = phi_b = 1


def primitives(oracle_mod, eos, phi, fluid):
    n = len(phi)
    sim = oracle_mod.OracleSim((n, 1, 1), precision="f32", eos=eos)
    sim._set_eos()
    field = np.zeros((n, 2), np.float32)
    field[:, 0] = phi
    u = np.ascontiguousarray(fluid, dtype=np.float32)
    prim = np.zeros((n, 4), np.float32)
    oracle_mod.lib().oracle_primitives_thermal_f32(oracle_mod._ptr(sim.P), oracle_mod._ptr(field),
                                                   oracle_mod._ptr(u), oracle_mod._ptr(prim))
    return prim


@pytest.mark.parametrize("which", ["max", "mass", "cubic", "zero"])
def test_inversion_recovers_fp64_states(oracle_mod, which):
    a, gmax, amax = bounds(oracle_mod)
    g, A = {"max": (gmax, amax), "mass": (gmax, 0.0), "cubic": (0.0, amax), "zero": (0.0, 0.0)}[which]
    rng = np.random.default_rng(7)
    n = 8192
    T = rng.uniform(0.75, 1.4, n)
    phi = rng.uniform(-0.05, 1.05, n)
    v = rng.normal(size=(n, 3))
    v *= (rng.uniform(0.0, 0.9, n) / np.linalg.norm(v, axis=1))[:, None]
    p = a / 3 * T**4 - 0.5 * g * T**2 * phi**2 + A / 3 * T * phi**3
    e = a * T**4 - 0.5 * g * T**2 * phi**2
    assert (p > a * T**4 / 12).all() and (p <= e).all()  # inside the validated range
    w = (e + p) / (1.0 - (v**2).sum(1))
    fluid = np.column_stack([w - p, w[:, None] * v])
    q = primitives(oracle_mod, ("thermal", g, A), phi, fluid)
    assert np.abs(q[:, 3] / p - 1.0).max() < 2e-5
    assert np.abs(q[:, :3] - v).max() < 2e-6


def run(oracle_mod, grid, eos, steps):
    sched = [(0.0, tuple(g / 2.0 for g in grid), 12.0)]
    s = oracle_mod.OracleSim(grid, schedule=sched, precision="f32", eos=eos)
    s.advance(10)
    e0 = s.diagnostics()["mean_energy_f64"]
    s.advance(steps)
    d = s.diagnostics()
    return s, d["mean_energy_f64"] / e0 - 1.0, d


def test_zero_coefficients_are_the_bag_model(oracle_mod):
    grid = (24, 24, 24)
    sb, drift_b, db = run(oracle_mod, grid, ("bag", 1.0, 0.0), 30)
    st, drift_t, dt = run(oracle_mod, grid, ("thermal", 0.0, 0.0), 30)
    fb, ub = sb.state()
    ft, ut = st.state()
    assert np.abs(ft - fb).max() < 1e-5
    assert np.abs(ut - ub).max() / np.abs(ub).max() < 1e-5
    assert dt["broken_fraction"] == pytest.approx(db["broken_fraction"], abs=1e-4)


def test_quiescent_state_is_a_fixed_point(oracle_mod):
    _, gmax, amax = bounds(oracle_mod)
    s = oracle_mod.OracleSim((12, 10, 9), precision="f32", eos=("thermal", gmax, amax))
    f0, u0 = s.state()
    s.advance(3)
    f1, u1 = s.state()
    assert f0.tobytes() == f1.tobytes() and u0.tobytes() == u1.tobytes()


def test_hot_broken_phase_feels_the_thermal_mass(oracle_mod):
    """phi = phi_b everywhere, T = 1.2 T_ref, A = 0: V'(phi_b) of the model
    vanishes, so with the friction eta pi the field sees
    pi(dt) = -gamma (T^2 - T_ref^2) phi_b (1 - exp(-eta dt)) / eta, up to the
    O(dt^2) change of phi."""
    a, gmax, _ = bounds(oracle_mod)
    g, T = gmax, 1.2
    grid = (8, 8, 8)
    s = oracle_mod.OracleSim(grid, precision="f32", eos=("thermal", g, 0.0))
    n = s.n
    field = np.zeros((n, 2), np.float32)
    field[:, 0] = 1.0
    fluid = np.zeros((n, 4), np.float32)
    fluid[:, 0] = a * T**4 - 0.5 * g * T**2  # at rest: E = e(T, phi_b)
    s.set_state(field, fluid)
    s.advance(1)
    f, _ = s.state()
    dt, eta = float(s.d["dt"]), float(s.model["eta"])
    want = -g * (T * T - 1.0) * (1.0 - np.exp(-eta * dt)) / eta
    assert np.ptp(f[:, 1]) == 0.0  # uniform
    assert f[0, 1] == pytest.approx(want, rel=5e-3)
    # the bag model has no such force
    b = oracle_mod.OracleSim(grid, precision="f32")
    b.set_state(field, fluid)
    b.advance(1)
    assert abs(b.state()[0][0, 1]) < 1e-3 * abs(want)


@pytest.mark.parametrize("which", ["mass", "both"])
def test_energy_conserved_like_the_bag_model(oracle_mod, which):
    _, gmax, amax = bounds(oracle_mod)
    g, A = (gmax, 0.0) if which == "mass" else (gmax, amax)
    grid = (32, 32, 32)
    _, drift_b, _ = run(oracle_mod, grid, ("bag", 1.0, 0.0), 100)
    _, drift_t, d = run(oracle_mod, grid, ("thermal", g, A), 100)
    assert np.isfinite(drift_t) and d["max_velocity"] < 0.5
    assert abs(drift_t) < 2.0 * abs(drift_b) + 2e-5
