import math
import os

import numpy as np

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M


def test_plot3d_roundtrip(tmp_path):
    v = M.trapezoid(5, 7, 6.0, 0.4, 15.0)
    p = str(tmp_path / "w.x")
    M.write_plot3d(p, v)
    r = M.read_plot3d(p, qc=False, dtype=np.float64)
    np.testing.assert_allclose(r[:3], v[:3], rtol=0, atol=1e-15)
    # the oracle reader agrees (quarter-chord shift included)
    np.testing.assert_allclose(M.read_plot3d(p, qc=True), O.read_plot3d(p, qc=True), rtol=0, atol=0)


def test_trapezoid_geometry():
    v = M.trapezoid(4, 8, 8.0, 0.5, 30.0)
    s = 8.0 * 1.5 / 4
    assert abs(v[1].max() - s) < 1e-12
    tip_chord = v[0, -1, -1] - v[0, 0, -1]
    assert abs(tip_chord - 0.5) < 1e-12
    assert abs(v[0, 0, -1] - s * math.tan(math.radians(30))) < 1e-12


def test_elliptic_geometry():
    v = M.elliptic(16, 16)
    assert abs(v[1, 0, -1] - 5.0) < 1e-12
    assert abs(v[0, -1, 0] - v[0, 0, 0] - 1.0) < 1e-12
    assert abs((v[0, 0, :] + 0.25 * (v[0, -1, :] - v[0, 0, :])) - 0.25).max() < 1e-12


def test_batch_cases_seeded():
    a = M.batch_cases(16)
    b = M.batch_cases(16)
    assert [c.params for c in a] == [c.params for c in b]
    for c in a:
        assert 4 <= c.nc <= 32 and 4 <= c.ns <= 64
        assert len(c.alphas) == 8 and np.all(np.abs(c.alphas) <= math.radians(8) + 1e-12)
