"""Shared fixtures: paths, builds, and the `gpu` marker.

Tests marked `gpu` need a CUDA device and call the library through its C
ABI; everything else runs on the CPU (the oracle, host logic and the
library's exported symbols).
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "bubble-simulation_gb300"
sys.path.insert(0, str(PKG))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def bubble():
    sys.path.insert(0, str(PKG))
    import build as pkg_build

    pkg_build.build()
    import bubble_gb300

    bubble_gb300.load()
    return bubble_gb300


@pytest.fixture(scope="session")
def gpu(bubble):
    """Skip-free GPU gate: a gpu test fails loudly without a device."""
    v = bubble.vram_query()
    assert v.capacity > 0
    return v
