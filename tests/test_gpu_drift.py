"""Energy drift of the FP32 forms against the FP64 CUDA oracle on the same
seeded lattice: the 128^3 default configuration (12 bubbles nucleated over
the first 40 time units, 1500 steps, reports every 100).  Drift is E/E0 - 1
with E0 the first report after every bubble is in (src/headless.rs:69-75).
Bar: each FP32 form's final drift within 1.5x of the FP64 drift (ratio in
[1/1.5, 1.5]).  With the reference's stage combine a0 U^n + a1 U1, FP32
totals (MIXED) gained a bias of 2.98e-8 per step from fl(1/3) + fl(2/3) != 1
(measured on GB300: FP64 3.50e-5, MIXED 6.66e-5, ratio 1.9); the fast
arithmetic now evaluates U^n + a1 (U1 - U^n)."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def drift_series(bubble, precision):
    spec = bubble.SimulationSpec(grid=(128, 128, 128), nucleation="uniform", bubbles=12, nucleation_duration=40.0,
                                 seed=1, precision=precision, math="fast")
    out, e0 = [], None
    with bubble.Simulation(spec) as sim:
        for _ in range(15):
            sim.advance(100)
            d = sim.diagnostics()
            if e0 is None and sim.remaining_bubbles() == 0:
                e0 = d.mean_energy_f64
            out.append(None if e0 is None else d.mean_energy_f64 / e0 - 1.0)
    return out


def test_drift_within_bounds_of_fp64(bubble, gpu):
    d64 = drift_series(bubble, "double")
    dm = drift_series(bubble, "mixed")
    dp = drift_series(bubble, "perturbation")
    print("final drift fp64 %.3e mixed %.3e perturbation %.3e" % (d64[-1], dm[-1], dp[-1]))
    assert abs(d64[-1]) > 1e-7
    for d in (dm, dp):
        assert 1 / 1.5 <= d[-1] / d64[-1] <= 1.5, (d[-1], d64[-1])
