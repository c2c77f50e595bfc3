"""The two forms of the fused stage kernel give identical bits.

For 16 x 16 FP32 tiles the stage kernel comes in two forms of the same
arithmetic (include/bubble_ext.h BUBBLE_STAGE_FORM_*):
- The register form keeps a column's z pipeline in registers, two CTAs per
  SM.
- The shared form reads the pipeline back from shared memory, three CTAs
  per SM.

AUTO picks by launch size; these tests force each form.

Checked here:
- Every FP32 form (plain, MIXED, perturbation, gamma-law and thermal
  equations of state) in both arithmetic modes, on shocked states and, for
  MIXED, on a state above gamma = 3, gives bit-identical results in both
  forms.
- The lattices have TMA-staged interior tiles and boundary tiles.
- The shared form gives the same bits under several z chunkings.
- The strict shared form matches the oracle directly.
"""
from __future__ import annotations

import numpy as np
import pytest

import make_golden

pytestmark = pytest.mark.gpu

GRIDS = [(48, 40, 36), (33, 17, 20)]
E_REF = 0.125  # e_ref of the default model


def _state(oracle_mod, grid, seed, kind, eos=None):
    sched = oracle_mod.make_schedule("centre", 1, 5.0, grid, 10.0, 1)
    kw = {"eos": eos} if eos else {}
    o = oracle_mod.OracleSim(grid, schedule=sched, precision="mixed" if kind == "mixed" else "f32", **kw)
    o.advance(4)
    if kind == "mixed":
        make_golden.relativistic_state(o, seed, 0.995)
    else:
        make_golden.perturbed_state(o, seed, 0.3)
    f, u = o.state()
    if kind == "perturbation":
        u = u.copy()
        u[:, 0] = (u[:, 0] - np.float32(o.d["e_ref"])).astype(np.float32)  # stored form: E - e_ref
    return f, u


def _run(bubble, grid, f0, u0, steps, form, math, precision="single", eos="bag", eos_param=(1.0, 0.0), lz=None):
    spec = bubble.SimulationSpec(grid=grid, bubbles=0, nucleation="centre", precision=precision, math=math,
                                 eos=eos, eos_param=eos_param)
    with bubble.Simulation(spec) as sim:
        sim.set_stage_form(form)
        if lz is not None:
            sim.set_tile(16, lz)
        sim.load_state(f0, u0)
        sim.advance(steps)
        return sim.copy_state()


def _same(a, b, what):
    bad = np.argwhere(np.asarray(a) != np.asarray(b))
    assert bad.size == 0, f"{what}: {len(bad)} differing values, first {bad[:3].tolist()}"


CASES = [
    # (state kind, precision, eos, eos_param, oracle eos)
    ("plain", "single", "bag", (1.0, 0.0), None),
    ("mixed", "mixed", "bag", (1.0, 0.0), None),
    ("perturbation", "perturbation", "bag", (1.0, 0.0), None),
    ("plain", "single", "gamma_law", (1.2, 0.05), ("gamma_law", 1.2, 0.05)),
    ("plain", "single", "thermal", (E_REF / 6.0, E_REF / np.sqrt(2.0)), ("thermal", E_REF / 6.0, E_REF / np.sqrt(2.0))),
]


@pytest.mark.parametrize("math", ["strict", "fast"])
@pytest.mark.parametrize("case", CASES, ids=[f"{c[1]}-{c[2]}" for c in CASES])
@pytest.mark.parametrize("grid", GRIDS)
def test_forms_bit_identical(bubble, oracle_mod, gpu, grid, case, math):
    kind, precision, eos, param, oeos = case
    f0, u0 = _state(oracle_mod, grid, 7, kind, oeos)
    kw = dict(precision=precision, eos=eos, eos_param=param)
    fr, ur = _run(bubble, grid, f0, u0, 6, "registers", math, **kw)
    fs, us = _run(bubble, grid, f0, u0, 6, "shared", math, **kw)
    assert np.isfinite(fr).all() and np.isfinite(ur).all()
    _same(fs, fr, "field")
    _same(us, ur, "fluid")


@pytest.mark.parametrize("math", ["strict", "fast"])
def test_shared_form_chunkings(bubble, oracle_mod, gpu, math):
    grid = (48, 40, 36)
    f0, u0 = _state(oracle_mod, grid, 8, "mixed")
    ref = _run(bubble, grid, f0, u0, 5, "shared", math, precision="mixed", lz=grid[2])
    for lz in (1, 5, 12):
        f, u = _run(bubble, grid, f0, u0, 5, "shared", math, precision="mixed", lz=lz)
        _same(f, ref[0], f"field lz {lz}")
        _same(u, ref[1], f"fluid lz {lz}")


def test_shared_form_strict_matches_oracle(bubble, oracle_mod, gpu):
    grid = (48, 40, 36)
    f0, u0 = _state(oracle_mod, grid, 9, "plain")
    o = oracle_mod.OracleSim(grid, precision="f32")
    o.set_state(f0, u0)
    o.advance(6)
    fo, uo = o.state()
    f, u = _run(bubble, grid, f0, u0, 6, "shared", "strict")
    _same(f, fo, "field")
    _same(u, uo, "fluid")


def test_unknown_form_is_rejected(bubble, gpu):
    with bubble.Simulation(bubble.SimulationSpec(grid=(16, 16, 16))) as sim:
        with pytest.raises(bubble.BubbleError) as e:
            bubble._lib.check(sim._L.bubble_ext_set_stage_form(sim._h, 3))
        assert e.value.code == bubble._lib.ERR_INVALID


def _stage_cost(n, lz, shared, sms):
    # the cost model of csrc/params.h column_stage_cost, restated for a cube
    tiles = ((n + 15) // 16) ** 2
    chunks = (n + lz - 1) // lz
    lz_eff = (n + chunks - 1) // chunks
    k, p = (3, 1.4) if shared else (2, 1.0)
    m = (tiles * chunks + sms - 1) // sms
    rounds = (m + k - 1) // k
    last = m - (rounds - 1) * k
    p_last = p if last == k else (0.65 * p if last == 1 else 0.8 * p)
    return ((rounds - 1) * p + p_last) * (lz_eff + 2)


def _model_chunk(n):
    """The cheapest chunk of an n^3 lattice under the stage cost model (ties
    to the longer chunk) for this device's SM count."""
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    best, best_lz = None, n
    for chunks in range(1, (n + 3) // 4 + 1):
        lz = (n + chunks - 1) // chunks
        c = min(_stage_cost(n, lz, False, sms), _stage_cost(n, lz, True, sms))
        if best is None or c < best * (1 - 1e-9):
            best, best_lz = c, lz
    return best_lz


@pytest.mark.parametrize("n", [32, 64, 96, 128, 160, 192, 256])
def test_default_chunk_follows_cost_model(bubble, gpu, n):
    """The default chunk of an FP32 lattice is the model's cheapest."""
    with bubble.Simulation(bubble.SimulationSpec(grid=(n, n, n), bubbles=1, nucleation="centre")) as sim:
        assert sim.tile() == (16, _model_chunk(n))


def test_auto_configuration_at_128_cubed(bubble, oracle_mod, gpu):
    """At 128^3 on 152 SMs the AUTO rule runs the shared form with 19-plane
    chunks (448 CTAs, TMA-staged interior tiles, uneven chunk ends). Strict MIXED there
    must match the oracle bit for bit, and fast MIXED must equal the register
    form with 32-plane chunks."""
    grid = (128, 128, 128)
    f0, u0 = _state(oracle_mod, grid, 10, "mixed")
    o = oracle_mod.OracleSim(grid, precision="mixed")
    o.set_state(f0, u0)
    o.advance(3)
    fo, uo = o.state()
    spec = bubble.SimulationSpec(grid=grid, bubbles=0, nucleation="centre", precision="mixed", math="strict")
    with bubble.Simulation(spec) as sim:
        assert sim.tile() == (16, _model_chunk(128))
        sim.load_state(f0, u0)
        sim.advance(3)
        f, u = sim.copy_state()
    _same(f, fo, "strict field")
    _same(u, uo, "strict fluid")
    auto = _run(bubble, grid, f0, u0, 3, "auto", "fast", precision="mixed")
    regs = _run(bubble, grid, f0, u0, 3, "registers", "fast", precision="mixed", lz=32)
    _same(auto[0], regs[0], "fast field")
    _same(auto[1], regs[1], "fast fluid")
