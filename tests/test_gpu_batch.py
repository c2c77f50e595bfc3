"""The batched form on the GPU: many lattices of uneven size in one
persistent, graph-captured launch.

Every lattice of a batch must evolve exactly as the plain per-lattice path
(include/bubble.h) evolves it: bit for bit in the strict mode (the same IEEE
operations in the same order, whatever kernel runs them), and with the same
grow/collapse outcome and a tolerance in the fast mode (separate kernel
instantiations may contract FMAs differently).  Nucleation events due in the
middle of a run split the persistent launches so each lattice stamps its
bubbles before the same step as the plain path.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def mixed_specs(bubble, n, math, seed=7, steps_events=False):
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n):
        edge = int(rng.choice([32, 48, 64, 96]))
        grid = (edge, edge, edge) if k % 3 else (edge, max(8, edge // 2), edge)
        model = bubble.Model(eta=float(np.exp(rng.uniform(np.log(0.02), np.log(1.0)))),
                             seed_value=float(rng.uniform(0.7, 1.5)))
        if steps_events:
            specs.append(bubble.SimulationSpec(model=model, grid=grid, nucleation="uniform", bubbles=2,
                                               nucleation_duration=3.0, seed=100 + k, math=math))
        else:
            specs.append(bubble.SimulationSpec(model=model, grid=grid, nucleation="centre", bubbles=1,
                                               seed=100 + k, math=math))
    return specs


def plain_run(bubble, spec, steps):
    with bubble.Simulation(spec) as sim:
        sim.advance(steps)
        return sim.copy_state(), sim.diagnostics()


@pytest.mark.parametrize("events", [False, True])
def test_batch_equals_plain_strict(bubble, gpu, events):
    specs = mixed_specs(bubble, 6, "strict", seed=3, steps_events=events)
    steps = 25
    with bubble.Batch(specs) as b:
        b.advance(10)
        b.advance(steps - 10)
        info = b.info()
        assert info["lattices"] == 6 and info["items"] > 0 and info["grid"] > 0
        got = [b.copy_state(k) for k in range(len(specs))]
        times = [b.time(k) for k in range(len(specs))]
    for k, spec in enumerate(specs):
        (f, u), _ = plain_run(bubble, spec, steps)
        assert np.array_equal(got[k][0], f), f"lattice {k} field"
        assert np.array_equal(got[k][1], u), f"lattice {k} fluid"
        with bubble.Simulation(spec) as sim:
            sim.advance(steps)
            assert times[k] == sim.time


@pytest.mark.parametrize("math", ["strict", "fast"])
def test_batch_solo_lattice_equals_plain(bubble, gpu, math):
    """A lattice that fills the GPU by itself (here 192^3) runs solo through
    the plain stage kernel with the plain path's chunk, beside the batched
    small lattices: it equals the plain path bit for bit in both arithmetic
    modes (same kernel, same chunk), events mid-run included."""
    model = bubble.Model(eta=0.1, seed_kind="cells", seed_value=12.0)
    big = bubble.SimulationSpec(model=model, grid=(192, 192, 192), nucleation="uniform", bubbles=4,
                                nucleation_duration=2.0, seed=9, math=math)
    specs = [big] + mixed_specs(bubble, 3, math, seed=5)
    steps = 12
    with bubble.Batch(specs) as b:
        b.advance(5)
        b.advance(steps - 5)
        got = [b.copy_state(k) for k in range(len(specs))]
        times = [b.time(k) for k in range(len(specs))]
    (f, u), _ = plain_run(bubble, big, steps)
    assert np.array_equal(got[0][0], f) and np.array_equal(got[0][1], u)
    with bubble.Simulation(big) as sim:
        sim.advance(steps)
        assert times[0] == sim.time
    if math == "strict":
        for k, spec in enumerate(specs[1:], start=1):
            (f, u), _ = plain_run(bubble, spec, steps)
            assert np.array_equal(got[k][0], f) and np.array_equal(got[k][1], u), k


def test_batch_fast_outcomes_match_plain(bubble, gpu):
    """The batched-ensemble workload in miniature: grow/collapse outcome of each
    run equals the plain path's, fields within 1e-4 after 300 steps."""
    specs = mixed_specs(bubble, 8, "fast", seed=11)
    steps = 300
    with bubble.Batch(specs) as b:
        b.advance(steps)
        diags = [b.diagnostics(k) for k in range(len(specs))]
        states = [b.copy_state(k) for k in range(len(specs))]
        assert b.info()["graph"] in (0, 1)
    for k, spec in enumerate(specs):
        (f, u), d = plain_run(bubble, spec, steps)
        assert (diags[k].broken_fraction > 0) == (d.broken_fraction > 0), k
        assert abs(diags[k].broken_fraction - d.broken_fraction) <= 2e-3
        for a, ref in ((states[k][0], f), (states[k][1], u)):
            scale = np.max(np.abs(ref), axis=0)
            assert np.max(np.max(np.abs(a - ref), axis=0) / scale) <= 1e-4, k


def test_batch_graph_replay_and_info(bubble, gpu):
    specs = mixed_specs(bubble, 4, "fast", seed=5)
    with bubble.Batch(specs, use_graph=True) as b:
        for _ in range(3):
            b.advance(5)
        info = b.info()
        assert info["graph"] == 1, info
        assert info["autotuned"] == 1
        assert info["cells"] == sum(s.grid[0] * s.grid[1] * s.grid[2] for s in specs)
    with bubble.Batch(specs, use_graph=False, autotune=False, max_grid=7) as b:
        b.advance(15)
        assert b.info()["grid"] == 7


def test_autotune_chunk(bubble, gpu):
    for edge in (32, 96):
        lz = bubble.autotune_chunk((edge, edge, edge), 8, "fast")
        assert 1 <= lz <= edge


def test_batch_rejects_mixed_modes(bubble, gpu):
    a = bubble.SimulationSpec(grid=(32, 32, 32), math="fast")
    c = bubble.SimulationSpec(grid=(32, 32, 32), math="strict")
    with pytest.raises(bubble.BubbleError):
        bubble.Batch([a, c])
    with pytest.raises(bubble.BubbleError):
        bubble.Batch([bubble.SimulationSpec(grid=(32, 32, 32), precision="double")])
