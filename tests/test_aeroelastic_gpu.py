"""Coupled aeroelastic pitch-plunge UVLM on the device (gbvlm_aero2dof_*,
the reference's tests/uvlm_2dof.cpp COUPLED loop) against the oracle's
restatement of the same loop (oracle.aero2dof_run, double aerodynamics and
structure).  Geometry: the reference's wing + flap pair (a chord-1
rectangle, span 40,000, split chordwise into a non-lifting front and a
lifting rear surface of 2 x 2 panels each), generated here; and one lifting
surface of 4 chordwise x 2 spanwise panels.  Parameters are the reference
run's (U_a = 7, above the linear flutter speed: the pitch grows into a
limit cycle through the cubic stiffness)."""
import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.aeroelastic import UVLM_2DOF, reference_vars

pytestmark = pytest.mark.gpu


def _wing_flap():
    v = M.rectangular(4, 2, 1.0, 40000.0).astype(np.float32)
    M.quarter_chord(v)
    return [np.ascontiguousarray(v[:, :3, :]), np.ascontiguousarray(v[:, 2:, :])], [0, 1]


def _single():
    v = M.rectangular(4, 2, 1.0, 40000.0).astype(np.float32)
    M.quarter_chord(v)
    return [v], [1]


@pytest.mark.parametrize("geom", ["wing_flap", "single"])
def test_aero2dof_matches_oracle(cuda, geom):
    surfaces, lifting = _wing_flap() if geom == "wing_flap" else _single()
    vars = reference_vars()
    t_final, steps = 100.0, 120
    ref = O.aero2dof_run(surfaces, lifting, vars, t_final, steps=steps)
    got = UVLM_2DOF(surfaces, lifting).run(vars, t_final, steps=steps)
    assert got["t_steps"] == ref["t_steps"] and abs(got["dt"] - ref["dt"]) < 1e-12
    amp = np.abs(ref["u"]).max(axis=0)
    err = np.abs(got["u"] - ref["u"]).max(axis=0)
    assert np.all(err <= 2e-4 * amp), (err, amp)
    famp = np.abs(ref["F"]).max(axis=0)
    ferr = np.abs(got["F"] - ref["F"]).max(axis=0)
    assert np.all(ferr <= 2e-3 * famp), (ferr, famp)
    # the same Newton effort, step by step, within one iteration
    assert np.abs(got["iters"].astype(int) - ref["iters"].astype(int)).max() <= 1


def test_aero2dof_resumes(cuda):
    """Advancing in two calls gives the same trajectory as one call."""
    surfaces, lifting = _wing_flap()
    vars = reference_vars()
    one = UVLM_2DOF(surfaces, lifting).run(vars, 40.0, steps=60)
    sim = UVLM_2DOF(surfaces, lifting)
    sim.start(vars, 40.0)
    sim.advance(25)
    sim.advance(35)
    two = sim.results()
    np.testing.assert_array_equal(two["u"], one["u"])
    np.testing.assert_array_equal(two["iters"], one["iters"])
