"""The allocation-free diagnostics entry point, bubble_diagnostics_noalloc.

It serves callers that cannot allocate device memory themselves (an engine
whose memory pool owns every byte, a real-time loop that must not allocate
mid-run): they pass their own device buffers and the reduction's scratch
comes from a static device array of the library.  This test calls it
through the C ABI on a lattice held by a Simulation and checks, on two
calls in a row, that it returns what bubble_diagnostics returns for the same
state: FP64 sums within 1e-12 relative, identical max|v| bits, broken count
and cell count.  This file is collected last so a failure here comes after
every other test has run; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(bubble, sim, model, precision, out_dev):
    L = bubble.load()
    field, fluid = ctypes.c_void_p(), ctypes.c_void_p()
    bubble._lib.check(L.bubble_ext_device_state(sim.handle, ctypes.byref(field), ctypes.byref(fluid)))
    grid = (ctypes.c_uint32 * 3)(*sim.grid)
    rc = L.bubble_diagnostics_noalloc(field, fluid, grid, ctypes.byref(model.c()),
                                      bubble._lib.PRECISION[precision], ctypes.c_void_p(out_dev),
                                      ctypes.c_void_p(sim.stream_ptr()))
    bubble._lib.check(rc)
    sim.synchronize()


@pytest.mark.parametrize("precision", ["single", "double"])
def test_noalloc_matches_diagnostics_on_two_calls(bubble, gpu, precision):
    import torch

    model = bubble.Model(seed_kind="cells", seed_value=10.0)
    spec = bubble.SimulationSpec(model=model, grid=(48, 40, 36), nucleation="simultaneous", bubbles=3,
                                 seed=4, precision=precision)
    # result buffer on the device: 4 doubles, 2 uint32, 1 uint64 = 48 bytes
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    with bubble.Simulation(spec) as sim:
        for call in range(2):
            sim.advance(7)
            want = sim.diagnostics()
            _noalloc(bubble, sim, model, precision, out.data_ptr())
            torch.cuda.synchronize()
            raw = out.cpu().numpy()
            sums = raw[:4]
            ints = raw[4:].view(np.uint32)
            max_v_bits, nonfinite, cells = int(ints[0]), int(ints[1]), int(raw[5:].view(np.uint64)[0])
            for got, ref in zip(sums, (want.sum_energy, want.sum_broken, want.sum_kinetic,
                                       want.sum_fluid_energy)):
                assert abs(got - ref) <= 1e-12 * abs(ref), (call, got, ref)
            assert np.uint32(max_v_bits).view(np.float32) == np.float32(want.max_velocity)
            assert nonfinite == 0
            assert cells == want.cells == 48 * 40 * 36


def test_noalloc_rejects_out_of_range_sizes(bubble, gpu):
    import torch

    L = bubble.load()
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    buf = torch.zeros(8, dtype=torch.float32, device="cuda")
    for grid in ((4, 16, 16), (16, 16, 4096)):
        rc = L.bubble_diagnostics_noalloc(ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()),
                                          (ctypes.c_uint32 * 3)(*grid), ctypes.byref(bubble.Model().c()), 0,
                                          ctypes.c_void_p(out.data_ptr()), None)
        assert rc == bubble._lib.ERR_INVALID
        assert "8..2048" in L.bubble_last_error().decode()
