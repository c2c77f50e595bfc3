"""The serving loop on the GPU (include/bubble_server.h).

Requests of different sizes and parameters arrive while others run, are
admitted against free device memory and advance together in the batched
launch.  The bar: each result is the same alone and in the mix -- bit for
bit in the strict mode (the per-lattice arithmetic does not depend on what
else is resident) -- and requests submitted while others are on the GPU are
admitted before those finish.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def request_specs(bubble, n, math, seed=9):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        edge = int(rng.choice([32, 48, 64]))
        model = bubble.Model(eta=float(np.exp(rng.uniform(np.log(0.02), np.log(1.0)))),
                             seed_value=float(rng.uniform(0.9, 1.5)))
        spec = bubble.SimulationSpec(model=model, grid=(edge, edge, edge), nucleation="uniform",
                                     bubbles=int(rng.integers(1, 4)), nucleation_duration=4.0, seed=50 + k,
                                     math=math)
        out.append((spec, int(rng.integers(20, 90))))
    return out


def alone(bubble, spec, steps):
    with bubble.Simulation(spec) as sim:
        sim.advance(steps)
        return sim.diagnostics()


def test_results_same_alone_and_in_the_mix(bubble, gpu):
    reqs = request_specs(bubble, 7, "strict")
    with bubble.Server(math="strict", chunk_steps=16) as srv:
        ids = [srv.submit(s, n) for s, n in reqs[:4]]
        srv.tick()
        srv.tick()  # the first four are resident and running
        ids += [srv.submit(s, n) for s, n in reqs[4:]]
        srv.run_until_idle()
        res = {r["id"]: r for r in srv.poll()}
        st = srv.stats()
    assert st["completed"] == st["submitted"] == 7 and st["queued"] == 0 and st["active"] == 0
    assert 0 < st["p50_latency_s"] <= st["p99_latency_s"]
    for i, (spec, steps) in zip(ids, reqs):
        r = res[i]
        assert r["status"] == 0 and r["steps"] == steps
        d = alone(bubble, spec, steps)
        for k in ("sum_energy", "sum_broken", "sum_kinetic", "sum_fluid_energy"):
            assert getattr(r["diag"], k) == getattr(d, k), (i, k)
        assert r["diag"].max_velocity == d.max_velocity


def test_late_requests_overlap_running_ones(bubble, gpu):
    reqs = request_specs(bubble, 3, "fast", seed=2)
    with bubble.Server(math="fast", chunk_steps=10) as srv:
        long_id = srv.submit(reqs[0][0], 200)
        srv.tick()
        late = [srv.submit(s, 30) for s, _ in reqs[1:]]
        srv.run_until_idle()
        res = {r["id"]: r for r in srv.poll()}
    for i in late:
        assert res[i]["admit_s"] < res[long_id]["done_s"]  # joined while the long one ran
        assert res[i]["done_s"] < res[long_id]["done_s"]


def test_oversized_request_is_refused(bubble, gpu):
    # 10 % above the device's capacity at 72 B/cell, within 2^32 - 1 cells
    v = bubble.vram_query()
    nz = min(int(1.1 * v.capacity / 72), 2**32 - 1) // (2048 * 2048)
    if 2048 * 2048 * nz * 72 <= v.capacity:
        pytest.skip("the device holds every lattice the 32-bit cell index allows")
    with bubble.Server() as srv:
        i = srv.submit(bubble.SimulationSpec(grid=(2048, 2048, nz)), 10)
        j = srv.submit(bubble.SimulationSpec(grid=(32, 32, 32), nucleation="centre", bubbles=1), 10)
        srv.run_until_idle()
        res = {r["id"]: r for r in srv.poll()}
    assert res[i]["status"] == bubble._lib.ERR_MEMORY
    assert res[j]["status"] == 0
