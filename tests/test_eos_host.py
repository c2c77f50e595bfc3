"""Equation-of-state selection on the CPU: the spec's policy and parameter
ranges (include/bubble.h BUBBLE_EOS_*), through the C ABI."""
from __future__ import annotations

import pytest


@pytest.mark.parametrize("eos,param,precision,ok", [
    ("bag", (1.0, 0.0), "single", True),
    ("bag", (1.0, 0.0), "double", True),
    ("bag_dof", (1.5, 0.0), "perturbation", True),
    ("bag_dof", (0.0, 0.0), "single", False),
    ("gamma_law", (4.0 / 3.0, 0.0), "single", True),
    ("gamma_law", (2.0, 0.1), "single", True),
    ("gamma_law", (2.1, 0.0), "single", False),   # acausal sound speed
    ("gamma_law", (1.0, 0.0), "single", False),   # c_s^2 = 0
    ("gamma_law", (1.5, 0.124), "single", False),  # e0 >= 0.99 e_ref (e_ref = 0.125)
    ("gamma_law", (1.5, -0.01), "single", False),
    ("gamma_law", (1.5, 0.0), "double", False),   # built for FP32 only
    # thermal potential, a = 0.125 at the default model: gamma <= a/6, A <= a/sqrt(2)
    ("thermal", (0.0, 0.0), "single", True),
    ("thermal", (0.02, 0.088), "single", True),
    ("thermal", (0.021, 0.0), "single", False),    # thermal mass above half the radiation pressure
    ("thermal", (0.0, 0.089), "single", False),    # p > e in the broken phase
    ("thermal", (-0.001, 0.0), "single", False),
    ("thermal", (0.01, -0.001), "single", False),
    ("thermal", (0.01, 0.01), "double", False),    # built for FP32 only
    ("thermal", (0.01, 0.01), "mixed", False),
])
def test_eos_validation(bubble, eos, param, precision, ok):
    spec = bubble.SimulationSpec(eos=eos, eos_param=param, precision=precision)
    msg = bubble.validate_eos(spec)
    assert (msg is None) == ok, msg


def test_spec_round_trip_keeps_eos(bubble):
    spec = bubble.SimulationSpec(eos="gamma_law", eos_param=(1.5, 0.02))
    back = bubble.SimulationSpec.from_c(spec.c())
    assert back.eos == "gamma_law" and back.eos_param == pytest.approx((1.5, 0.02))


def test_spec_round_trip_keeps_thermal(bubble):
    spec = bubble.SimulationSpec(eos="thermal", eos_param=(0.015, 0.05))
    back = bubble.SimulationSpec.from_c(spec.c())
    assert back.eos == "thermal" and back.eos_param == pytest.approx((0.015, 0.05))
