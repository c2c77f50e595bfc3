"""The allocation-free diagnostics entry point, bubble_diagnostics_noalloc.

It serves callers that cannot allocate device memory themselves (an engine
whose memory pool owns every byte, a real-time loop that must not allocate
mid-run): they pass their own device buffers and the lattice's spec, and the
reduction's scratch comes from a static device array of the library.  This
test calls it through the C ABI on a lattice held by a Simulation and
checks, on two calls in a row, that it returns what bubble_diagnostics
returns for the same state: FP64 sums within 1e-12 relative, identical
max|v| bits, broken count and cell count.  It covers every precision form
and equation of state the library steps (the MIXED case on a state with
cells above gamma = 3, where its FP64 recovery runs).  This file is
collected last so a failure here comes after every other test has run; it
also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import make_golden

pytestmark = pytest.mark.gpu

A_RAD = 0.125  # e_ref / T_ref^4 of the default model

FORMS = [
    ("single", "bag", (1.0, 0.0)),
    ("mixed", "bag", (1.0, 0.0)),
    ("double", "bag", (1.0, 0.0)),
    ("perturbation", "bag", (1.0, 0.0)),
    ("single", "gamma_law", (1.5, 0.01)),
    ("single", "thermal", (A_RAD / 6.0, A_RAD / np.sqrt(2.0))),
]


def _noalloc(bubble, sim, spec, out_dev):
    L = bubble.load()
    field, fluid = ctypes.c_void_p(), ctypes.c_void_p()
    bubble._lib.check(L.bubble_ext_device_state(sim.handle, ctypes.byref(field), ctypes.byref(fluid)))
    c = spec.c()
    rc = L.bubble_diagnostics_noalloc(field, fluid, ctypes.byref(c), ctypes.c_void_p(out_dev),
                                      ctypes.c_void_p(sim.stream_ptr()))
    bubble._lib.check(rc)
    sim.synchronize()


@pytest.mark.parametrize("precision,eos,param", FORMS)
def test_noalloc_matches_diagnostics_on_two_calls(bubble, gpu, oracle_mod, precision, eos, param):
    import torch

    grid = (48, 40, 36)
    model = bubble.Model(seed_kind="cells", seed_value=10.0)
    spec = bubble.SimulationSpec(model=model, grid=grid, nucleation="simultaneous", bubbles=3, seed=4,
                                 precision=precision, eos=eos, eos_param=param)
    # result buffer on the device: 4 doubles, 2 uint32, 1 uint64 = 48 bytes
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    with bubble.Simulation(spec) as sim:
        if precision == "mixed":
            # a ball moving at up to |v| = 0.995: the FP64 recovery runs
            o = oracle_mod.OracleSim(grid, precision="mixed")
            assert make_golden.relativistic_state(o, 21, 0.995) > 20
            sim.load_state(*o.state())
        for call in range(2):
            sim.advance(7)
            want = sim.diagnostics()
            _noalloc(bubble, sim, spec, out.data_ptr())
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
            if precision == "mixed":
                assert want.max_velocity > 0.943


def test_noalloc_rejects_out_of_range_sizes(bubble, gpu):
    import torch

    L = bubble.load()
    out = torch.zeros(6, dtype=torch.float64, device="cuda")
    buf = torch.zeros(8, dtype=torch.float32, device="cuda")
    for grid in ((4, 16, 16), (16, 16, 4096)):
        spec = bubble.SimulationSpec(grid=grid).c()
        rc = L.bubble_diagnostics_noalloc(ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()),
                                          ctypes.byref(spec), ctypes.c_void_p(out.data_ptr()), None)
        assert rc == bubble._lib.ERR_INVALID
        assert "8..2048" in L.bubble_last_error().decode()
    # a spec bubble_create would refuse (the gamma law is FP32 only)
    spec = bubble.SimulationSpec(grid=(16, 16, 16), precision="double", eos="gamma_law",
                                 eos_param=(1.5, 0.0)).c()
    rc = L.bubble_diagnostics_noalloc(ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(buf.data_ptr()),
                                      ctypes.byref(spec), ctypes.c_void_p(out.data_ptr()), None)
    assert rc == bubble._lib.ERR_INVALID
