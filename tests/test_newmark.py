"""The oracle's Newmark-beta restatement (oracle/oracle.py newmark_*) against
golden vectors produced by the reference's own scripts/newmark.py on the
3-DOF system of its tests/newmark.cpp (tests/golden/make_newmark_golden.py)."""
import json
import os

import numpy as np

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "newmark_3dof.json")


def test_oracle_newmark_matches_reference_script():
    with open(GOLD) as f:
        g = json.load(f)
    u, v, a = O.newmark_linear(np.array(g["M"]), np.array(g["C"]), np.array(g["K"]), np.array(g["u0"]),
                               np.array(g["v0"]), g["dt"], g["steps"])
    for name, x in (("u", u), ("v", v), ("a", a)):
        ref = np.array(g[name])
        assert np.abs(x - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), name


def test_newmark_trapezoidal_rule_conserves_energy_without_damping():
    # beta = 1/4, gamma = 1/2 (the reference's defaults) conserve the energy of an undamped system
    K = np.array([[2.0, -1.0], [-1.0, 2.0]])
    M = np.eye(2)
    u, v, a = O.newmark_linear(M, np.zeros((2, 2)), K, np.array([0.1, 0.0]), np.zeros(2), 0.05, 2000)
    e = 0.5 * np.einsum("ti,ij,tj->t", v, M, v) + 0.5 * np.einsum("ti,ij,tj->t", u, K, u)
    assert np.abs(e - e[0]).max() <= 1e-12
