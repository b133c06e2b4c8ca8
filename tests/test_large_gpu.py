"""Large steady path: one AIC, many right-hand sides (the 64-alpha sweep of
the 16,384-panel workload, here on a 32 x 32 elliptic wing so the double
oracle finishes quickly), against the full double solve at 1e-5."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("refine", [0, 1])
def test_elliptic_sweep_64_alphas(cuda, refine):
    v = M.elliptic(24, 32).astype(np.float32)
    M.quarter_chord(v)
    al = np.radians(np.linspace(-10.0, 10.0, 64))
    case = M.Case(v, al, {})
    bs = BatchSolver([case], mode="shared", refine=refine)
    bs.set_inputs(pack_verts([case]), pack_alphas([case]))
    bs.run(want_gamma=True)
    co, gam = bs.results(gamma=True)
    ref = O.vlm_shared([v.astype(np.float64)], al)
    cls = np.array([float(r["cl"]) for r in ref])
    guard = 1e-3 * np.abs(cls).max()
    for k, r in enumerate(ref):
        cl = float(r["cl"])
        assert abs(co[k, 0] - cl) <= 1e-5 * max(abs(cl), guard), (k, co[k, 0], cl)
        g = np.concatenate([x.ravel() for x in r["gamma"]])
        assert np.linalg.norm(gam[k] - g) <= 1e-5 * np.linalg.norm(g) + 1e-9
