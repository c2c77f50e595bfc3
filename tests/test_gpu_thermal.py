"""Thermal potential on the GPU (include/bubble.h BUBBLE_EOS_THERMAL,
docs/EOS.md:120-150).

* strict arithmetic bit-identical with the oracle's FP32 restatement
  (stepping, diagnostics with the field's V(phi, 0), and the vis pack's
  temperature from the inverted p(T, phi)), across the validated parameter
  range;
* gamma = A = 0 reproduces the bag model to FP32 rounding in both
  arithmetic modes, and the fast mode tracks the strict one;
* the quiescent state is a fixed point and energy is conserved as for the
  bag model (the reference's acceptance checks for a new EOS,
  docs/EOS.md:156-169);
* the policy runs on the default kernel path only and refuses the others.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A_RAD = 0.125  # e_ref / T_ref^4 of the default model
G_MAX, A_MAX = A_RAD / 6.0, A_RAD / np.sqrt(2.0)


def shocked_state(oracle_mod, grid, seed, eos, amp=0.3):
    import make_golden

    sched = oracle_mod.make_schedule("centre", 1, 5.0, grid, 10.0, 1)
    o = oracle_mod.OracleSim(grid, schedule=sched, precision="f32", eos=eos)
    o.advance(4)
    make_golden.perturbed_state(o, seed, amp)
    return o.state()


def sim(bubble, grid, param, math="strict", eos="thermal", model=None):
    spec = bubble.SimulationSpec(model=model or bubble.Model(), grid=grid, nucleation="centre", bubbles=0,
                                 precision="single", math=math, eos=eos, eos_param=param)
    return bubble.Simulation(spec)


PARAMS = [(G_MAX, A_MAX), (G_MAX, 0.0), (0.0, 0.05), (0.0, 0.0)]


@pytest.mark.parametrize("param", PARAMS)
@pytest.mark.parametrize("grid,seed", [((9, 11, 13), 1), ((40, 20, 18), 2)])
def test_thermal_strict_bit_exact(bubble, oracle_mod, gpu, param, grid, seed):
    eos = ("thermal",) + param
    f0, u0 = shocked_state(oracle_mod, grid, seed, eos)
    o = oracle_mod.OracleSim(grid, precision="f32", eos=eos)
    o.set_state(f0, u0)
    o.advance(5)
    fr, ur = o.state()
    assert np.isfinite(fr).all() and np.isfinite(ur).all()
    dr = o.diagnostics()
    with sim(bubble, grid, param) as s:
        s.load_state(f0, u0)
        s.advance(5)
        f, u = s.copy_state()
        d = s.diagnostics()
    assert f.tobytes() == fr.tobytes(), np.abs(f - fr).max()
    assert u.tobytes() == ur.tobytes(), np.abs(u - ur).max()
    assert d.sum_energy == pytest.approx(dr["sum_energy"], rel=1e-12)
    assert d.max_velocity == dr["max_velocity"]


@pytest.mark.parametrize("param", [(G_MAX, A_MAX), (G_MAX, 0.0)])
def test_thermal_vis_pack_bit_exact(bubble, oracle_mod, gpu, param):
    grid = (40, 20, 18)
    eos = ("thermal",) + param
    f0, u0 = shocked_state(oracle_mod, grid, 2, eos)
    o = oracle_mod.OracleSim(grid, precision="f32", eos=eos)
    o.set_state(f0, u0)
    want = o.visualise()
    with sim(bubble, grid, param) as s:
        s.load_state(f0, u0)
        s.visualise()
        got = s.vis_texture()
    assert got.tobytes() == want.tobytes()


def test_thermal_zero_coefficients_and_fast_mode(bubble, gpu):
    grid = (40, 40, 40)
    model = bubble.Model(seed_kind="cells", seed_value=10.0)
    out = {}
    for eos, param in (("bag", (1.0, 0.0)), ("thermal", (0.0, 0.0)), ("thermal", (G_MAX, A_MAX))):
        for math in ("strict", "fast"):
            with sim(bubble, grid, param, math=math, eos=eos, model=model) as s:
                s.reset([(0.0, (20.0, 20.0, 20.0), 10.0)])
                s.advance(60)
                out[eos, param, math] = s.copy_state()
    for math in ("strict", "fast"):
        fb, ub = out["bag", (1.0, 0.0), math]
        fz, uz = out["thermal", (0.0, 0.0), math]
        assert np.abs(fz - fb).max() < 1e-5
        assert np.abs(uz - ub).max() / np.abs(ub).max() < 1e-5
    fs, us = out["thermal", (G_MAX, A_MAX), "strict"]
    ff, uf = out["thermal", (G_MAX, A_MAX), "fast"]
    assert np.isfinite(ff).all() and np.isfinite(uf).all()
    assert np.abs(ff - fs).max() < 2e-4
    assert np.abs(uf - us).max() / np.abs(us).max() < 2e-4


@pytest.mark.parametrize("math", ["strict", "fast"])
def test_thermal_quiescent_and_conservation(bubble, gpu, math):
    with sim(bubble, (24, 24, 24), (G_MAX, A_MAX), math=math) as s:
        f0, u0 = s.copy_state()
        s.advance(5)
        f, u = s.copy_state()
        assert f.tobytes() == f0.tobytes() and u.tobytes() == u0.tobytes()
    model = bubble.Model(seed_kind="cells", seed_value=12.0)
    drift = {}
    for eos, param in (("bag", (1.0, 0.0)), ("thermal", (G_MAX, A_MAX))):
        with sim(bubble, (48, 48, 48), param, math=math, eos=eos, model=model) as s:
            s.reset([(0.0, (24.0, 24.0, 24.0), 12.0)])
            s.advance(10)
            e0 = s.diagnostics().mean_energy_f64
            s.advance(150)
            d = s.diagnostics()
        assert np.isfinite(d.max_velocity) and d.max_velocity > 0
        drift[eos] = d.mean_energy_f64 / e0 - 1.0
    assert abs(drift["thermal"]) < 5e-4
    assert abs(drift["thermal"]) < 2.0 * abs(drift["bag"]) + 2e-5


def test_thermal_rejects_other_paths(bubble, gpu):
    with sim(bubble, (16, 16, 16), (0.01, 0.01), math="fast") as s:
        with pytest.raises(bubble.BubbleError):
            s.set_tile(4, 16)
        s.set_path("reference")
        with pytest.raises(bubble.BubbleError):
            s.advance(1)
