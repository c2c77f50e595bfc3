"""The simulation driver's API on the GPU, after src/gpu/gpu_tests.rs.

Resize grow/shrink/non-cubic with the stepping check of
gpu_tests.rs:60-116, memory accounting (:171-189), a rejected resize leaving
the state intact (:193-214), plus the failure paths this build adds:
admission refusal, a forced allocation failure, an invalid model, and the
record_steps / advance nucleation semantics (src/gpu/sim.rs:827-879).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def spec(bubble, grid, **kw):
    base = dict(model=bubble.Model(), grid=grid, nucleation="simultaneous", bubbles=1,
                nucleation_duration=10.0, seed=1)
    base.update(kw)
    return bubble.SimulationSpec(**base)


def step_and_check(sim, what):
    sim.advance(8)
    d = sim.diagnostics()
    assert np.isfinite(d.mean_energy), what
    assert np.isfinite(d.max_velocity), what
    assert d.mean_energy > 0.0, what
    assert 0.0 <= d.broken_fraction <= 1.0, what
    assert d.max_velocity < 1.0, what


def test_resize_rebuilds_a_working_simulation(bubble, gpu):
    with bubble.Simulation(spec(bubble, (64, 64, 64))) as sim:
        assert sim.cell_count() == 64 ** 3
        step_and_check(sim, "initial 64^3")
        sim.resize((96, 96, 96))
        assert sim.grid == (96, 96, 96) and sim.cell_count() == 96 ** 3
        assert sim.time == 0.0
        step_and_check(sim, "grown to 96^3")
        sim.resize((32, 32, 32))
        assert sim.cell_count() == 32 ** 3
        step_and_check(sim, "shrunk to 32^3")
        sim.resize((48, 32, 72))
        assert sim.grid == (48, 32, 72) and sim.cell_count() == 48 * 32 * 72
        step_and_check(sim, "non-cubic 48x32x72")


def test_memory_accounting(bubble, gpu):
    for grid in [(64, 64, 64), (128, 128, 128), (48, 32, 72)]:
        with bubble.Simulation(spec(bubble, grid)) as sim:
            predicted = bubble.lattice_bytes(grid)
            actual = sim.device_memory_bytes()
            assert abs(actual - predicted) / predicted < 0.01 or actual - predicted < 200_000


def test_resize_release_before_allocate(bubble, gpu):
    # Free memory after shrinking returns to the level of the smaller lattice.
    v0 = bubble.vram_query()
    with bubble.Simulation(spec(bubble, (256, 256, 256))) as sim:
        v1 = bubble.vram_query()
        assert v1.used - v0.used >= bubble.lattice_bytes((256,) * 3) * 0.99
        sim.resize((64, 64, 64))
        v2 = bubble.vram_query()
        assert v2.used - v0.used < bubble.lattice_bytes((256,) * 3) * 0.1


def test_rejected_resize_leaves_state_intact(bubble, gpu):
    with bubble.Simulation(spec(bubble, (64, 64, 64))) as sim:
        sim.advance(3)
        f0, u0 = sim.copy_state()
        with pytest.raises(bubble.BubbleError) as e:
            sim.resize((4, 64, 64))
        assert e.value.code == bubble._lib.ERR_INVALID and "at least 8 cells" in e.value.message
        assert sim.grid == (64, 64, 64) and sim.steps == 3
        f1, u1 = sim.copy_state()
        assert np.array_equal(f0, f1) and np.array_equal(u0, u1)
        step_and_check(sim, "after rejected resize")


def test_admission_refuses_oversized_lattice(bubble, gpu):
    # a lattice 10 % above the device's capacity at 72 B/cell, within the
    # 2^32 - 1 cells the stage kernels index (2048 x 2048 x nz)
    v = bubble.vram_query()
    cells = min(int(1.1 * v.capacity / 72), 2**32 - 1)
    nz = cells // (2048 * 2048)
    if 2048 * 2048 * nz * 72 <= v.capacity:
        pytest.skip("the device holds every lattice the 32-bit cell index allows")
    with pytest.raises(bubble.BubbleError) as e:
        bubble.Simulation(spec(bubble, (2048, 2048, nz)))
    assert e.value.code == bubble._lib.ERR_MEMORY
    with bubble.Simulation(spec(bubble, (32, 32, 32))) as sim:  # still usable
        step_and_check(sim, "after refusal")


def test_forced_allocation_failure(bubble, gpu):
    bubble.load().bubble_ext_inject_allocation_failure()
    with pytest.raises(bubble.BubbleError) as e:
        bubble.Simulation(spec(bubble, (32, 32, 32)))
    assert e.value.code == bubble._lib.ERR_MEMORY
    with bubble.Simulation(spec(bubble, (32, 32, 32))) as sim:
        step_and_check(sim, "after a failed allocation")


def test_set_model(bubble, gpu):
    with bubble.Simulation(spec(bubble, (32, 32, 32))) as sim:
        with pytest.raises(bubble.BubbleError) as e:
            sim.set_model(bubble.Model(cfl=0.9))
        assert e.value.code == bubble._lib.ERR_INVALID
        assert abs(sim.model.cfl - 0.2) < 1e-7
        sim.set_model(bubble.Model(eta=0.05))
        assert abs(sim.model.eta - 0.05) < 1e-7
        step_and_check(sim, "after set_model")


def test_record_steps_vs_advance_nucleation(bubble, gpu):
    sched = [(0.0, (10.0, 10.0, 10.0), 6.0), (0.5, (30.0, 30.0, 30.0), 6.0)]
    with bubble.Simulation(spec(bubble, (40, 40, 40), bubbles=0)) as a:
        a.reset(sched)
        a.record_steps(5)  # nucleation once (t = 0), then 5 steps
        assert a.remaining_bubbles() == 1 and abs(a.time - 1.0) < 1e-6
        a.record_steps(0)
        assert a.remaining_bubbles() == 0
    with bubble.Simulation(spec(bubble, (40, 40, 40), bubbles=0)) as b:
        b.reset(sched)
        b.advance(5)  # checked before every step: second bubble at t = 0.6
        assert b.remaining_bubbles() == 0


def test_nucleate_now(bubble, gpu):
    with bubble.Simulation(spec(bubble, (48, 48, 48), bubbles=0)) as sim:
        sim.advance(2)
        assert sim.remaining_bubbles() == 0
        sim.nucleate_now(42)
        assert sim.remaining_bubbles() == 1
        sim.advance(1)
        assert sim.remaining_bubbles() == 0
        assert sim.diagnostics().broken_fraction > 0.0


def test_state_round_trip_and_external_stream(bubble, gpu):
    import torch

    with bubble.Simulation(spec(bubble, (40, 24, 16))) as sim:
        sim.advance(4)
        f, u = sim.copy_state()
        s = torch.cuda.Stream()
        sim.set_stream(s.cuda_stream)
        sim.load_state(f, u)
        f2, u2 = sim.copy_state()
        assert np.array_equal(f, f2) and np.array_equal(u, u2)
        sim.advance(2)
        sim.set_stream(None)
        step_and_check(sim, "after stream switch")


def test_precisions_agree(bubble, gpu):
    # FP32 rounding floor of this 60-step run against FP64 is ~1.3e-4 (pi).
    out = {}
    for prec in ("single", "mixed", "double"):
        with bubble.Simulation(spec(bubble, (48, 48, 48), precision=prec,
                                    model=bubble.Model(seed_kind="cells", seed_value=14.0))) as sim:
            sim.advance(60)
            out[prec] = sim.copy_state()
    for prec in ("single", "mixed"):
        for a, b in zip(out[prec], out["double"]):
            scale = np.max(np.abs(b), axis=0)
            assert np.max(np.max(np.abs(a - b), axis=0) / scale) < 5e-4, prec
