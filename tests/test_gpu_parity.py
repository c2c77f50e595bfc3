"""Parity of the CUDA kernels with the oracle, through the C ABI.

Bars (stated per test):
  * strict FP32 path (fused and reference-structured): bit-identical with the
    FP32 oracle;
  * FP64 path: bit-identical with the FP64 oracle;
  * fast FP32 path: normwise max relative error <= 1e-5 per component
    (max|gpu - oracle| / max|oracle|), after up to 100 steps;
  * nucleation: bit-identical (FP32 and FP64);
  * diagnostics: FP64 sums within 1e-12 relative, max|v| and broken count exact.
At the full 512^3 size, where the oracle is too slow, size-independent
properties are checked: the fused kernel equals the reference-structured
kernel bit for bit, periodic translation commutes with stepping, and the
quiescent state is a fixed point.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = ["odd", "tile_partial", "flat"]


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN / "cases.npz"))


def spec_for(bubble, grid, precision="single", math="strict", nucleation="simultaneous",
             bubbles=0, model=None, seed=1):
    return bubble.SimulationSpec(model=model or bubble.Model(), grid=tuple(int(g) for g in grid),
                                 nucleation=nucleation, bubbles=bubbles, precision=precision,
                                 math=math, seed=seed)


def gpu_run(bubble, grid, field0, fluid0, steps, precision="single", math="strict", path="fused",
            tile=None):
    with bubble.Simulation(spec_for(bubble, grid, precision, math)) as sim:
        if path != "fused":
            sim.set_path(path)
        if tile:
            sim.set_tile(*tile)
        sim.load_state(field0, fluid0)
        sim.advance(steps)
        return sim.copy_state()


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b), axis=0)
    scale[scale == 0] = 1.0
    return float(np.max(np.max(np.abs(a - b), axis=0) / scale))


def assert_bit_equal(a, b, what):
    a = np.asarray(a)
    b = np.asarray(b)
    bad = np.argwhere(a != b)
    assert bad.size == 0, f"{what}: {len(bad)} differing values, first at {bad[:3].tolist()}: " \
                          f"{a[tuple(bad[0])]} vs {b[tuple(bad[0])]}"


# ---- committed golden fixtures ---------------------------------------------
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("path", ["fused", "reference"])
def test_strict_fp32_bit_exact_vs_golden(bubble, gpu, golden, case, path):
    grid = golden[f"{case}_grid"]
    steps = int(golden[f"{case}_steps"])
    f, u = gpu_run(bubble, grid, golden[f"{case}_f32_field0"], golden[f"{case}_f32_fluid0"], steps,
                   path=path)
    assert_bit_equal(f, golden[f"{case}_f32_field"], f"{case} field")
    assert_bit_equal(u, golden[f"{case}_f32_fluid"], f"{case} fluid")


@pytest.mark.parametrize("case", CASES)
def test_fp64_bit_exact_vs_golden(bubble, gpu, golden, case):
    grid = golden[f"{case}_grid"]
    steps = int(golden[f"{case}_steps"])
    f, u = gpu_run(bubble, grid, golden[f"{case}_f64_field0"], golden[f"{case}_f64_fluid0"], steps,
                   precision="double")
    assert_bit_equal(f, golden[f"{case}_f64_field"], f"{case} field")
    assert_bit_equal(u, golden[f"{case}_f64_fluid"], f"{case} fluid")


@pytest.mark.parametrize("case", CASES)
def test_fast_fp32_within_tolerance_vs_golden(bubble, gpu, golden, case):
    grid = golden[f"{case}_grid"]
    steps = int(golden[f"{case}_steps"])
    f, u = gpu_run(bubble, grid, golden[f"{case}_f32_field0"], golden[f"{case}_f32_fluid0"], steps,
                   math="fast")
    assert rel_err(f, golden[f"{case}_f32_field"]) <= 1e-5
    assert rel_err(u, golden[f"{case}_f32_fluid"]) <= 1e-5


# ---- live oracle on fresh seeded inputs ------------------------------------
@pytest.mark.parametrize("seed", [11, 12])
@pytest.mark.parametrize("grid", [(16, 8, 24), (33, 17, 10)])
def test_strict_and_f64_vs_live_oracle(bubble, gpu, oracle_mod, seed, grid):
    import make_golden

    out = {}
    for prec in ("f32", "f64"):
        sched = oracle_mod.make_schedule("simultaneous", 3, 4.0, grid, 1.0, seed)
        sim = oracle_mod.OracleSim(grid, schedule=sched, precision=prec)
        sim.record_nucleation()
        make_golden.perturbed_state(sim, seed, 0.35)
        f0, u0 = sim.state()
        sim.advance(6)
        out[prec] = (f0, u0) + sim.state()
    f0, u0, fr, ur = out["f32"]
    f, u = gpu_run(bubble, grid, f0, u0, 6)
    assert_bit_equal(f, fr, "f32 field")
    assert_bit_equal(u, ur, "f32 fluid")
    f0, u0, fr, ur = out["f64"]
    f, u = gpu_run(bubble, grid, f0, u0, 6, precision="double")
    assert_bit_equal(f, fr, "f64 field")
    assert_bit_equal(u, ur, "f64 fluid")


def test_100_steps_single_bubble_against_fp64(bubble, gpu, oracle_mod):
    """Per-cell fields after 100 steps of a 40^3 single-bubble run.

    The strict FP32 path equals the FP32 oracle bit for bit.  Against the
    FP64 CUDA oracle (itself bit-identical with the FP64 CPU oracle), the
    reference-order FP32 arithmetic is off by up to ~8e-5 (phi) and ~3e-5
    (Z), the FP32 rounding floor of this case; the fast path must be no less
    accurate: per component, err(fast) <= 1.5 err(strict) + 1e-6.  The fast
    stage combine is U^n + a1 (U1 - U^n), whose weights sum to 1 in binary32,
    and the strict one the reference's a0 U^n + a1 U1, whose third-stage
    weights sum to 1 + 2^-25, so the two paths differ by up to the sum of
    their distances to FP64, not by less than either.
    """
    grid = (40, 40, 40)
    sched = oracle_mod.make_schedule("centre", 1, 9.0, grid, 10.0, 1)
    o = oracle_mod.OracleSim(grid, schedule=sched)
    o.advance(100)
    fo, uo = o.state()
    model = bubble.Model(seed_kind="cells", seed_value=9.0)
    out = {}
    for prec, mode in (("single", "strict"), ("single", "fast"), ("double", "strict")):
        spec = spec_for(bubble, grid, precision=prec, math=mode, nucleation="centre", bubbles=1, model=model)
        with bubble.Simulation(spec) as sim:
            sim.advance(100)
            out[(prec, mode)] = sim.copy_state()
    fs, us = out[("single", "strict")]
    ff, uf = out[("single", "fast")]
    fd, ud = out[("double", "strict")]
    assert_bit_equal(fs, fo, "strict field")
    assert_bit_equal(us, uo, "strict fluid")

    def comp_err(a, b):
        a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
        return np.max(np.abs(a - b), axis=0) / np.max(np.abs(b), axis=0)

    for fast, strict, ref in ((ff, fs, fd), (uf, us, ud)):
        e_fast, e_strict = comp_err(fast, ref), comp_err(strict, ref)
        assert np.all(e_fast <= 1.5 * e_strict + 1e-6), (e_fast, e_strict)
        assert np.all(comp_err(fast, strict) <= e_fast + e_strict + 1e-6), (e_fast, e_strict)


# ---- nucleation and diagnostics --------------------------------------------
@pytest.mark.parametrize("precision", ["single", "double"])
def test_nucleation_bit_exact(bubble, gpu, oracle_mod, precision):
    grid = (40, 36, 32)
    sched = oracle_mod.make_schedule("simultaneous", 9, 6.5, grid, 1.0, 5)
    o = oracle_mod.OracleSim(grid, schedule=sched, precision="f32" if precision == "single" else "f64")
    o.record_nucleation()
    spec = spec_for(bubble, grid, precision, nucleation="simultaneous", bubbles=9,
                    model=bubble.Model(seed_kind="cells", seed_value=6.5), seed=5)
    with bubble.Simulation(spec) as sim:
        assert [tuple(map(float, e[1])) for e in sim.schedule()] == \
            [tuple(map(float, e[1])) for e in sched]
        sim.record_steps(0)
        f, u = sim.copy_state()
        assert sim.remaining_bubbles() == 0
    fo, uo = o.state()
    assert_bit_equal(f, fo, "nucleated field")
    assert_bit_equal(u, uo, "fluid untouched")
    assert (f[:, 0] > 0.5).sum() > 0


@pytest.mark.parametrize("grid", [(8, 8, 8), (2048, 8, 8), (8, 2048, 8), (8, 8, 2048), (33, 9, 200)])
def test_extreme_shapes_bit_exact(bubble, gpu, oracle_mod, grid):
    """The axis limits (8 and 2048 cells) and lopsided boxes: the smallest
    lattice the 5-point stencil allows, one 2048-cell axis with the others at
    the minimum (one x tile of 2048 columns; 256 y tiles; one column of 2048
    planes), and an odd shape no tile divides.  Strict FP32 and FP64 against
    the oracle, bit for bit, after nucleation and 4 steps."""
    for prec, p in (("single", "f32"), ("double", "f64")):
        sched = oracle_mod.make_schedule("simultaneous", 2, 3.0, grid, 1.0, 4)
        o = oracle_mod.OracleSim(grid, schedule=sched, precision=p)
        o.advance(4)
        fo, uo = o.state()
        spec = spec_for(bubble, grid, prec, nucleation="simultaneous", bubbles=2,
                        model=bubble.Model(seed_kind="cells", seed_value=3.0), seed=4)
        with bubble.Simulation(spec) as sim:
            sim.advance(4)
            f, u = sim.copy_state()
        assert_bit_equal(f, fo, f"{p} field {grid}")
        assert_bit_equal(u, uo, f"{p} fluid {grid}")


@pytest.mark.parametrize("precision", ["single", "double"])
def test_nucleation_culling_bit_exact(bubble, gpu, oracle_mod, precision):
    """The brick-culled nucleation kernel against the oracle's loop over the
    whole batch: 300 bubbles (three launches of <= 128), a grid that is no
    multiple of the 32 x 8 x 8 brick, small radii so most bricks keep few
    bubbles, and a field that is negative everywhere beforehand, so the max
    with the far field (exactly 0) must reach every cell."""
    grid = (45, 37, 29)
    p = "f32" if precision == "single" else "f64"
    sched = oracle_mod.make_schedule("simultaneous", 300, 2.0, grid, 1.0, 11)
    o = oracle_mod.OracleSim(grid, schedule=sched, precision=p)
    f0, u0 = o.state()
    rng = np.random.default_rng(3)
    f0 = f0.copy()
    f0[:, 0] = -np.abs(rng.standard_normal(len(f0))).astype(f0.dtype) * f0.dtype.type(0.01)
    o.set_state(f0, u0)
    o.record_nucleation()
    spec = spec_for(bubble, grid, precision, nucleation="simultaneous", bubbles=300,
                    model=bubble.Model(seed_kind="cells", seed_value=2.0), seed=11)
    with bubble.Simulation(spec) as sim:
        sim.load_state(f0, u0)
        sim.record_steps(0)
        f, _ = sim.copy_state()
    fo, _ = o.state()
    assert_bit_equal(f, fo, "nucleated field")
    assert (f[:, 0] >= 0).all()


@pytest.mark.parametrize("precision", ["single", "double"])
def test_diagnostics_match_oracle(bubble, gpu, golden, oracle_mod, precision):
    case = "tile_partial"
    p = "f32" if precision == "single" else "f64"
    grid = tuple(int(g) for g in golden[f"{case}_grid"])
    o = oracle_mod.OracleSim(grid, precision=p)
    o.set_state(golden[f"{case}_{p}_field"], golden[f"{case}_{p}_fluid"])
    do = o.diagnostics()
    with bubble.Simulation(spec_for(bubble, grid, precision)) as sim:
        sim.load_state(golden[f"{case}_{p}_field"], golden[f"{case}_{p}_fluid"])
        d = sim.diagnostics()
    for k in ("sum_energy", "sum_kinetic", "sum_fluid_energy"):
        assert abs(getattr(d, k) - do[k]) <= 1e-12 * abs(do[k]), k
    assert d.sum_broken == do["sum_broken"]
    assert np.float32(d.max_velocity) == np.float32(do["max_velocity"])


def test_nonfinite_state_is_reported(bubble, gpu):
    # A NaN in E alone would be hidden by max(E, e_floor) in the energy term
    # (IEEE maxNum, as in the reference); the check also scans the raw state.
    grid = (16, 16, 16)
    for comp, where in ((0, "fluid"), (1, "field"), (3, "fluid")):
        with bubble.Simulation(spec_for(bubble, grid)) as sim:
            f, u = sim.copy_state()
            (u if where == "fluid" else f)[123, comp] = np.nan if comp != 3 else np.inf
            sim.load_state(f, u)
            with pytest.raises(bubble.BubbleError) as e:
                sim.diagnostics()
            assert e.value.code == bubble._lib.ERR_NONFINITE


# ---- tile shapes and the full-size properties ------------------------------
def test_tile_shapes_agree(bubble, gpu, golden):
    """In the strict arithmetic every tile shape and z chunking gives the same
    bits (each operation is one IEEE rounding whatever kernel instantiation
    runs it).  In the fast arithmetic every z chunking of one instantiation
    gives identical bits; the tile shapes (16 x 16, 32 x 8, 32 x 4) are
    separate instantiations whose FMA contraction may differ, so they agree
    within the fast-path bar, 1e-5 relative (measured: 1.6e-6 after 5 steps
    of this shocked case)."""
    case = "tile_partial"
    grid = golden[f"{case}_grid"]
    f0, u0 = golden[f"{case}_f32_field0"], golden[f"{case}_f32_fluid0"]

    def run(math, tile):
        with bubble.Simulation(spec_for(bubble, grid, "single", math)) as sim:
            sim.set_tile(*tile)
            sim.load_state(f0, u0)
            sim.advance(5)
            return sim.copy_state()

    ref = run("strict", (16, 64))
    for tile in [(16, 1), (16, 3), (16, 7), (8, 64), (8, 3)]:
        got = run("strict", tile)
        assert_bit_equal(got[0], ref[0], f"strict field tile {tile}")
        assert_bit_equal(got[1], ref[1], f"strict fluid tile {tile}")
    for ty in (16, 8):
        ref = run("fast", (ty, 64))
        for lz in (1, 3, 7):
            got = run("fast", (ty, lz))
            assert_bit_equal(got[0], ref[0], f"fast field tile {(ty, lz)}")
            assert_bit_equal(got[1], ref[1], f"fast fluid tile {(ty, lz)}")
    ref = run("fast", (16, 64))
    for tile in [(8, 64), (4, 3), (4, 64)]:
        got = run("fast", tile)
        assert rel_err(got[0], ref[0]) <= 1e-5 and rel_err(got[1], ref[1]) <= 1e-5, tile


@pytest.mark.parametrize("precision", ["mixed", "perturbation"])
def test_fast_forms_chunkings_agree(bubble, gpu, golden, precision):
    """The fast primitive recovery rounds explicitly, so the chunk prologue
    and the z-march give the same bits and every z chunking of the fast
    MIXED and perturbation forms agrees bit for bit too."""
    case = "tile_partial"
    grid = golden[f"{case}_grid"]
    f0 = np.array(golden[f"{case}_f32_field0"])
    u0 = np.array(golden[f"{case}_f32_fluid0"])
    if precision == "perturbation":  # stored form: E - e_ref
        e_ref = np.float32(bubble.derived(bubble.Model())["e_ref"])
        u0 = u0.copy()
        u0[..., 0] = (u0[..., 0] - e_ref).astype(np.float32)

    def run(lz):
        with bubble.Simulation(spec_for(bubble, grid, precision, "fast")) as sim:
            sim.set_tile(16, lz)
            sim.load_state(f0, u0)
            sim.advance(5)
            return sim.copy_state()

    ref = run(64)
    for lz in (1, 3, 7):
        got = run(lz)
        assert_bit_equal(got[0], ref[0], f"{precision} field lz {lz}")
        assert_bit_equal(got[1], ref[1], f"{precision} fluid lz {lz}")


def test_fp64_chunkings_agree(bubble, gpu, golden):
    case = "odd"
    grid = golden[f"{case}_grid"]
    f0, u0 = golden[f"{case}_f64_field0"], golden[f"{case}_f64_fluid0"]
    ref = gpu_run(bubble, grid, f0, u0, 4, precision="double", tile=(16, 64))
    for tile in [(16, 1), (16, 5), (4, 1), (4, 64)]:
        got = gpu_run(bubble, grid, f0, u0, 4, precision="double", tile=tile)
        assert_bit_equal(got[0], ref[0], f"field tile {tile}")
        assert_bit_equal(got[1], ref[1], f"fluid tile {tile}")


def _bubbly_state(bubble, grid, nb, seed):
    spec = spec_for(bubble, grid, nucleation="simultaneous", bubbles=nb, seed=seed,
                    model=bubble.Model(seed_kind="cells", seed_value=10.0))
    with bubble.Simulation(spec) as sim:
        sim.advance(30)
        return sim.copy_state()


@pytest.mark.parametrize("grid", [(512, 512, 512), (96, 80, 72)])
def test_fused_equals_reference_structure_at_size(bubble, gpu, grid):
    f0, u0 = _bubbly_state(bubble, grid, 8, 3)
    a = gpu_run(bubble, grid, f0, u0, 2, path="fused")
    b = gpu_run(bubble, grid, f0, u0, 2, path="reference")
    assert_bit_equal(a[0], b[0], "field")
    assert_bit_equal(a[1], b[1], "fluid")


@pytest.mark.parametrize("math", ["fast", "strict"])
def test_translation_commutes_with_stepping_at_512(bubble, gpu, math):
    grid = (512, 512, 512)
    f0, u0 = _bubbly_state(bubble, grid, 6, 9)
    shift = (37, -101, 250)  # cells along x, y, z
    def roll(a):
        a = a.reshape(grid[2], grid[1], grid[0], -1)
        return np.roll(a, (shift[2], shift[1], shift[0]), axis=(0, 1, 2)).reshape(-1, a.shape[-1])
    a = gpu_run(bubble, grid, f0, u0, 2, math=math)
    b = gpu_run(bubble, grid, roll(f0), roll(u0), 2, math=math)
    assert_bit_equal(roll(a[0]), b[0], "field")
    assert_bit_equal(roll(a[1]), b[1], "fluid")


def test_quiescent_fixed_point_at_512(bubble, gpu):
    grid = (512, 512, 512)
    with bubble.Simulation(spec_for(bubble, grid, math="fast")) as sim:
        f0, u0 = sim.copy_state()
        sim.advance(3)
        f, u = sim.copy_state()
        d = sim.diagnostics()
    assert_bit_equal(f, f0, "field")
    assert_bit_equal(u, u0, "fluid")
    assert d.max_velocity == 0.0 and d.broken_fraction == 0.0
