"""Nonlinear VLM oracle (strip-wise correction toward a 2D polar,
vlm/src/vlm.cpp:153-295) against the reference's own known answers,
tests/nlvlm_curves.cpp: the 5 x 200 "infinite" rectangle at alpha = 19 deg
with three lift curves (two Spallart curves with stall, the thin-airfoil
line) tabulated at 100 angles in [0, 20] deg; CL within 1 % of the curve."""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M


def spallart(cl0, a0, a1, cla0, cla1):
    return lambda a: cla0 * a + 0.5 * (cl0 - cla1 * a) * (1.0 + math.erf((a - a0) / a1))


CURVES = {
    "spallart1": spallart(1.2, 0.28, 0.02, 2 * math.pi, 2 * math.pi),
    "spallart2": spallart(0.72, 0.28, 0.04, 2 * math.pi, 1.5 * math.pi),
    "polar": lambda a: 2 * math.pi * a,
}


def rectangle_5x200():
    v = M.rectangular(5, 200, 1.0, 40000.0).astype(np.float32)
    M.quarter_chord(v)
    return v


def polar_table(curve):
    a = np.linspace(0.0, math.radians(20.0), 100).astype(np.float32)
    return a, np.array([curve(float(x)) for x in a], np.float32)


@pytest.mark.parametrize("name", sorted(CURVES))
def test_oracle_lift_curves(name):
    a, cl = polar_table(CURVES[name])
    alpha = math.radians(19.0)
    r = O.nlvlm_run([rectangle_5x200()], alpha, a, cl)
    exact = CURVES[name](alpha)
    assert abs(r["cl"] - exact) / exact < 0.01, (name, r["cl"], exact)
    assert r["err"] <= 1e-5 and r["iters"] <= 100


def test_akima_nodes_and_lines():
    x = np.linspace(-0.3, 0.4, 23).astype(np.float64)
    y = np.sin(3 * x) + x
    tab = O.akima_table(x, y, np.float64)
    for xi, yi in zip(x, y):
        assert abs(O.akima_eval(tab, xi) - yi) < 1e-14
    lin = O.akima_table(x, 2.0 * x - 1.0, np.float64)
    for q in (-0.5, -0.3, -0.11, 0.05, 0.4, 0.7):  # inside and outside the table
        assert abs(O.akima_eval(lin, q) - (2.0 * q - 1.0)) < 1e-12


def test_reference_mesh_is_the_generated_one():
    from tests import ref_fixtures as R
    v = R.mesh("infinite_rectangular_5x200")
    assert np.abs(v - rectangle_5x200()).max() == 0.0
