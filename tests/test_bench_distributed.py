"""The N > 1 bookkeeping of bench.py on the CPU, with world_size-2 gloo
process groups (127.0.0.1): the whole-job clock is the slowest rank's time,
and under torchrun the reference arm runs and prints on rank 0 alone."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, times, out: str):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    got = bench.max_over_ranks(times[rank], dist, "cpu")
    dist.barrier()
    with open(f"{out}.{rank}", "w") as f:
        f.write(repr(got))
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    times = [12.5, 31.25]
    out = str(tmp_path / "r")
    mp.start_processes(_rank, args=(2, free_port(), times, out), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        assert float(open(f"{out}.{r}").read()) == max(times)


def test_max_over_ranks_single_rank():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(7.0, None, "cpu") == 7.0


def test_reference_arm_under_torchrun(oracle_mod, tmp_path):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--workload", "default128", "--steps", "1", "--warmup", "0", "--gpus", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] in ("port", "reference")
