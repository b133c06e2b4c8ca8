"""Nonlinear VLM on the GPU (gbvlm_nlvlm_*, the NLVLM mirror in
tinyvlm_gb300.vlm) against the oracle's restatement of vlm.cpp:153-295 and
the reference's known answers (tests/nlvlm_curves.cpp: CL within 1 % of the
lift curve at 19 deg).  Float (the reference's precision) against the
double oracle within 2e-4 of CL; double against it within 5e-8; strip
angles and iteration counts alike."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.vlm import NLVLM, Database, FlowData, WingProfile

from .test_nlvlm import CURVES, polar_table, rectangle_5x200

pytestmark = pytest.mark.gpu


def _db(curve):
    a, cl = polar_table(curve)
    db = Database()
    db.profiles.append(WingProfile(a, cl))
    db.profiles_pos.append(0.0)
    return db, a, cl


@pytest.mark.parametrize("name", sorted(CURVES))
def test_reference_lift_curves(cuda, name):
    db, a, cl = _db(CURVES[name])
    alpha = math.radians(19.0)
    sim = NLVLM("gb300", [rectangle_5x200()])
    res = sim.run(FlowData(alpha), db)
    exact = CURVES[name](alpha)
    assert abs(res.cl - exact) / exact < 0.01, (name, res.cl, exact)
    ref = O.nlvlm_run([rectangle_5x200()], alpha, a, cl, dtype=np.float64)
    assert abs(res.cl - ref["cl"]) <= 2e-4 * abs(ref["cl"]), (res.cl, ref["cl"])
    assert sim.iters == ref["iters"]


def test_two_surfaces_double_against_oracle(cuda):
    """A swept, tapered wing split in two surfaces: the strips converge to
    different angles; the double path matches the double oracle strip by strip."""
    v = M.trapezoid(6, 24, 7.0, 0.45, 25.0)
    M.quarter_chord(v)
    ns = v.shape[2] - 1
    parts = [np.ascontiguousarray(v[:, :, : ns // 2 + 1]), np.ascontiguousarray(v[:, :, ns // 2:])]
    db, a, cl = _db(CURVES["spallart2"])
    alpha = math.radians(18.0)  # past the curve's knee: the strips settle at different angles (5 iterations)
    ref = O.nlvlm_run(parts, alpha, a, cl, dtype=np.float64, beta=math.radians(2.0))
    sim = NLVLM("gb300", parts, precision=64)
    res = sim.run(FlowData(alpha, beta=math.radians(2.0)), db)
    # the double kernels evaluate the Biot-Savart law in a cancellation-free
    # arrangement, ~1e-9 from the oracle's restatement of the reference's
    # FP64 kernel (the steady double path is held to 1e-8); the strip
    # corrections carry that through a few iterations
    assert abs(res.cl - ref["cl"]) <= 5e-8 * abs(ref["cl"]), (res.cl, ref["cl"])
    assert sim.iters == ref["iters"]
    for g, r in zip(sim.strip_alpha, ref["strip_alpha"]):
        np.testing.assert_allclose(g, r, rtol=0, atol=1e-6)  # the strip angles are returned as float
    assert np.ptp(np.concatenate(ref["strip_alpha"])) > 5e-3  # the strips really differ
    f32 = NLVLM("gb300", parts).run(FlowData(alpha, beta=math.radians(2.0)), db)
    assert abs(f32.cl - ref["cl"]) <= 2e-4 * abs(ref["cl"])


def test_zero_iterations_and_rerun(cuda):
    db, a, cl = _db(CURVES["polar"])
    sim = NLVLM("gb300", [rectangle_5x200()], precision=64)
    first = sim.run(FlowData(math.radians(5.0)), db).cl
    sim.max_iter = 0
    sim.run(FlowData(math.radians(5.0)), db)  # no iteration: the loads of the last circulation
    assert sim.iters == 0
    sim.max_iter = 100
    again = sim.run(FlowData(math.radians(5.0)), db).cl
    assert again == first
