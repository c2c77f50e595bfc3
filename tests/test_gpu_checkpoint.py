"""Checkpoint and resume on the GPU: a run saved at step k and resumed
reaches bit for bit the states of the uninterrupted run, with nucleation
events still pending at the checkpoint."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import PKG

pytestmark = pytest.mark.gpu


def spec(bubble, grid=(48, 40, 36), precision="single", math="fast"):
    return bubble.SimulationSpec(grid=grid, nucleation="exponential", bubbles=6, nucleation_duration=12.0, seed=5,
                                 precision=precision, math=math,
                                 model=bubble.Model(seed_kind="cells", seed_value=8.0))


@pytest.mark.parametrize("precision,math", [("single", "fast"), ("mixed", "strict"), ("double", "fast")])
def test_resume_is_bit_exact(bubble, gpu, tmp_path, precision, math):
    path = tmp_path / "run.ckpt"
    with bubble.Simulation(spec(bubble, precision=precision, math=math)) as a:
        a.advance(20)
        assert a.remaining_bubbles() > 0  # events still pending at the checkpoint
        a.save_checkpoint(str(path))
        t20 = a.time
        a.advance(40)
        fa, ua = a.copy_state()
        da = a.diagnostics()
        ta, sa, ra = a.time, a.steps, a.remaining_bubbles()
    with bubble.Simulation.from_checkpoint(str(path)) as b:
        assert b.steps == 20 and b.time == t20
        b.advance(40)
        fb, ub = b.copy_state()
        db = b.diagnostics()
        assert (b.time, b.steps, b.remaining_bubbles()) == (ta, sa, ra)
    assert fa.tobytes() == fb.tobytes() and ua.tobytes() == ub.tobytes()
    assert (da.sum_energy, da.sum_broken, da.sum_kinetic, da.max_velocity) == \
        (db.sum_energy, db.sum_broken, db.sum_kinetic, db.max_velocity)


def test_restore_into_other_grid_and_layout_checks(bubble, gpu, tmp_path):
    path = tmp_path / "r.ckpt"
    with bubble.Simulation(spec(bubble)) as a:
        a.advance(5)
        a.save_checkpoint(str(path))
        f5, u5 = a.copy_state()
    with bubble.Simulation(spec(bubble, grid=(16, 16, 16))) as b:
        b.restore_checkpoint(str(path))  # resized to the checkpoint's grid
        assert b.grid == (48, 40, 36) and b.steps == 5
        f, u = b.copy_state()
        assert f.tobytes() == f5.tobytes() and u.tobytes() == u5.tobytes()
    with bubble.Simulation(spec(bubble, grid=(16, 16, 16), precision="double")) as c:
        with pytest.raises(bubble.BubbleError):
            c.restore_checkpoint(str(path))  # FP32 file into an FP64 simulation
        assert c.grid == (16, 16, 16)  # unchanged


def test_cli_save_and_resume(bubble, gpu, tmp_path):
    cli = str(PKG / "lib" / "bubble-sim")
    ck = tmp_path / "cli.ckpt"
    common = ["--grid", "40", "--bubbles", "4", "--nucleation-duration", "10", "--report-every", "10"]
    full = subprocess.run([cli, *common, "--headless", "50"], capture_output=True, text=True, timeout=300)
    first = subprocess.run([cli, *common, "--headless", "20", "--save-checkpoint", str(ck)], capture_output=True,
                           text=True, timeout=300)
    second = subprocess.run([cli, "--resume", str(ck), "--headless", "30", "--report-every", "10"],
                            capture_output=True, text=True, timeout=300)
    for r in (full, first, second):
        assert r.returncode == 0, r.stderr
    def rows(out):  # the report table's rows (not the throughput line)
        return [ln.split()[:6] for ln in out.splitlines() if ln.strip()[:1].isdigit() and "steps in" not in ln]

    # the resumed run's report rows (absolute step numbers) equal the full run's last three
    assert rows(second.stdout) == rows(full.stdout)[-3:]
    assert rows(first.stdout) == rows(full.stdout)[:2]
