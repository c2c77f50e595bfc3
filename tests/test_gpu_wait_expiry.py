"""Bounded device waits that run out, and the error the host reads back.

The reference stops a run whose diagnostics go bad (src/headless.rs:63-67);
here every wait a kernel makes on the device is bounded as well, so a wait
that would never end becomes an error status instead of a hung GPU.  These
tests make the two kinds of wait run out without any faulty access:

  * the stage kernel's TMA plane wait: a test hook arms, in every CTA that
    stages planes through TMA, the first plane's mbarrier for bytes that no
    copy delivers and issues no copy for that plane, with a short limit
    (2^20 SM cycles, about half a millisecond);
  * the persistent batch kernel's grid barrier: a test hook sets the
    barrier's release count one above the grid, so no arrival releases it.

Each time the host must read BUBBLE_ERR_TIMEOUT, clear it, and the same
device must then run fresh work bit-identically with the oracle or with the
plain path: the context stays usable.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHIFT = 20


def _oracle_run(oracle_mod, grid, steps):
    sched = oracle_mod.make_schedule("simultaneous", 2, 4.0, grid, 1.0, 4)
    o = oracle_mod.OracleSim(grid, schedule=sched)
    o.advance(steps)
    return o.state()


def _spec(bubble, grid, math="strict"):
    return bubble.SimulationSpec(model=bubble.Model(seed_kind="cells", seed_value=4.0), grid=grid,
                                 nucleation="simultaneous", bubbles=2, seed=4, math=math)


def test_stage_wait_expires_and_reports_timeout(bubble, gpu, oracle_mod):
    L = bubble.load()
    # 96 x 48 has 16 x 16 column tiles whose halo lies inside the lattice:
    # they stage by TMA
    grid = (96, 48, 24)
    with bubble.Simulation(_spec(bubble, grid)) as sim:
        sim.advance(2)
        sim.synchronize()
        bubble._lib.check(L.bubble_ext_test_expire_stage_wait(sim.handle, 64, SHIFT))
        sim.advance(1)
        with pytest.raises(bubble.BubbleError) as e:
            sim.synchronize()
        assert e.value.code == bubble._lib.ERR_TIMEOUT
        sim.synchronize()  # the status was read and cleared
        assert L.bubble_ext_test_expire_stage_wait(sim.handle, 0, SHIFT) == bubble._lib.ERR_INVALID
    # the device still runs: a fresh lattice matches the oracle bit for bit
    fo, uo = _oracle_run(oracle_mod, grid, 3)
    with bubble.Simulation(_spec(bubble, grid)) as sim:
        sim.advance(3)
        f, u = sim.copy_state()
    assert np.array_equal(f, fo) and np.array_equal(u, uo)


def test_batch_barrier_expires_and_reports_timeout(bubble, gpu):
    L = bubble.load()
    specs = [_spec(bubble, (32, 32, 32)), _spec(bubble, (48, 40, 32)), _spec(bubble, (32, 24, 40))]
    with bubble.Batch(specs, autotune=False) as b:
        b.advance(1)
        bubble._lib.check(L.bubble_ext_test_expire_batch_barrier(b._h, SHIFT))
        b.advance(2)
        with pytest.raises(bubble.BubbleError) as e:
            b.diagnostics(0)
        assert e.value.code == bubble._lib.ERR_TIMEOUT
        b.diagnostics(0)  # the status was read and cleared
    # the device still runs: a fresh batch equals the plain path bit for bit
    with bubble.Batch(specs, autotune=False) as b:
        b.advance(4)
        got = [b.copy_state(k) for k in range(len(specs))]
    for k, spec in enumerate(specs):
        with bubble.Simulation(spec) as sim:
            sim.advance(4)
            f, u = sim.copy_state()
        assert np.array_equal(got[k][0], f) and np.array_equal(got[k][1], u), k
