"""The oracle's MIXED precision form, pinned on the CPU.

MIXED keeps the FP32 state and kernels but redoes the primitive recovery in
FP64 wherever the FP32 recovery gives v^2 > 8/9 (Lorentz factor above 3),
the inversion the reference's precision plan moves to FP64
(docs/PRECISION.md:150-152 of the reference).  Its restatement is pinned
here against the FP64 oracle: on every cell above the threshold the MIXED
primitive must equal the FP64 oracle's primitive of the widened FP32 state,
rounded once (the same IEEE double operations); on every other cell it must
equal the FP32 primitive.  The perturbation form's fallback is pinned the
same way against a numpy FP64 restatement of its inversion.
"""
from __future__ import annotations

import numpy as np
import pytest

import make_golden

GRIDS = [(16, 8, 24), (24, 24, 24)]


def _relativistic(oracle_mod, grid, precision, seed=11, v_peak=0.995):
    sched = oracle_mod.make_schedule("simultaneous", 2, 3.0, grid, 1.0, 4)
    sim = oracle_mod.OracleSim(grid, schedule=sched, precision=precision)
    sim.record_nucleation()
    n_hot = make_golden.relativistic_state(sim, seed, v_peak)
    return sim, n_hot


def _prims(sim):
    sim.diagnostics()  # runs the primitives pass over the current slot
    return sim.prim.copy()


@pytest.mark.parametrize("grid", GRIDS)
def test_mixed_recovery_is_fp64_above_gamma3(oracle_mod, grid):
    s32, n_hot = _relativistic(oracle_mod, grid, "f32")
    assert n_hot > 20, "the state must hold cells above gamma = 3"
    f0, u0 = s32.state()
    q32 = _prims(s32)
    smx = oracle_mod.OracleSim(grid, precision="mixed")
    smx.set_state(f0, u0)
    qmx = _prims(smx)
    s64 = oracle_mod.OracleSim(grid, precision="f64")
    s64.set_state(f0.astype(np.float64), u0.astype(np.float64))
    q64 = _prims(s64)
    v2 = (q32[:, 0] * q32[:, 0] + q32[:, 1] * q32[:, 1]) + q32[:, 2] * q32[:, 2]  # FP32, kernel order
    hot = v2 > np.float32(8.0) / np.float32(9.0)
    assert hot.sum() == n_hot
    np.testing.assert_array_equal(qmx[hot], q64[hot].astype(np.float32))
    np.testing.assert_array_equal(qmx[~hot], q32[~hot])
    # the fallback is more accurate where it applies: pressure against FP64
    e32 = np.abs(q32[hot, 3].astype(np.float64) - q64[hot, 3]) / q64[hot, 3]
    emx = np.abs(qmx[hot, 3].astype(np.float64) - q64[hot, 3]) / q64[hot, 3]
    assert emx.max() <= 6e-8 < e32.max()


def test_perturbation_form_has_the_fp64_fallback(oracle_mod):
    grid = (24, 24, 24)
    sp, n_hot = _relativistic(oracle_mod, grid, "pert")
    assert n_hot > 20
    q = _prims(sp)
    _, u = sp.state()
    d = oracle_mod.derived(oracle_mod.DEFAULT_MODEL)
    e_ref = np.float32(d["e_ref"])
    e_floor = np.float64(np.float32(d["e_floor"] - e_ref))
    p_floor = np.float64(np.float32(d["p_floor"] - np.float32(e_ref / np.float32(3.0))))
    z_max = np.float64(d["z_max"])
    u64 = u.astype(np.float64)
    de = np.maximum(u64[:, 0], e_floor)
    e_lab = np.float64(e_ref) + de
    z = u64[:, 1:].copy()
    zlen = np.sqrt((z[:, 0] * z[:, 0] + z[:, 1] * z[:, 1]) + z[:, 2] * z[:, 2])
    zcap = z_max * e_lab
    over = zlen > zcap
    z[over] *= (zcap[over] / np.maximum(zlen[over], 1e-30))[:, None]
    z2 = (z[:, 0] * z[:, 0] + z[:, 1] * z[:, 1]) + z[:, 2] * z[:, 2]
    sq = np.sqrt(np.maximum(4.0 * e_lab * e_lab - 3.0 * z2, 0.0))
    dp = np.maximum(de / 3.0 - z2 / (sq + 2.0 * e_lab), p_floor)
    den = np.maximum(e_lab + np.float64(np.float32(e_ref / np.float32(3.0))) + dp, 1e-30)
    ref = np.stack([z[:, 0] / den, z[:, 1] / den, z[:, 2] / den, dp], axis=1).astype(np.float32)
    # cells well above gamma = 3 (v^2 > 0.9, so the FP32 pre-check flags
    # them too) are recovered in FP64, bit-identical with the restatement
    v2 = (q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1]) + q[:, 2] * q[:, 2]
    hot = v2 > np.float32(0.9)
    assert hot.sum() > 20
    np.testing.assert_array_equal(q[hot], ref[hot])


def test_mixed_equals_single_below_gamma3(oracle_mod):
    """With no cell above gamma = 3 the MIXED form is the FP32 form bit for bit."""
    grid = (16, 12, 10)
    out = {}
    for prec in ("f32", "mixed"):
        sched = oracle_mod.make_schedule("simultaneous", 2, 3.0, grid, 1.0, 4)
        sim = oracle_mod.OracleSim(grid, schedule=sched, precision=prec)
        sim.record_nucleation()
        make_golden.perturbed_state(sim, 5, 0.3)
        sim.advance(4)
        out[prec] = sim.state()
    np.testing.assert_array_equal(out["f32"][0], out["mixed"][0])
    np.testing.assert_array_equal(out["f32"][1], out["mixed"][1])
