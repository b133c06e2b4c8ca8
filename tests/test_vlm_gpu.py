"""Steady VLM end to end on the GPU (plain per-solve path, float and double)
against the oracle and against the reference's known-answer tests."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import wing
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.vlm import VLM, FlowData

pytestmark = pytest.mark.gpu


def _cases():
    a = M.rectangular(3, 4, 1.0, 20000.0, 0.0).astype(np.float32)
    b = M.rectangular(3, 4, 1.0, 20000.0, 20000.0).astype(np.float32)
    M.quarter_chord(a)
    M.quarter_chord(b)
    return {"trap": [wing("trap", 6, 10)], "ellip": [wing("ellip", 8, 8)], "split": [a, b]}


@pytest.mark.parametrize("name", ["trap", "ellip", "split"])
@pytest.mark.parametrize("prec", [32, 64])
def test_vlm_matches_oracle(cuda, name, prec):
    surf = _cases()[name]
    sim = VLM("gb300", surf, precision=prec)
    npd = np.float32 if prec == 32 else np.float64
    for adeg in (0.0, 3.0, 10.0):
        al = math.radians(adeg)
        ref = O.vlm_run([s.astype(npd) for s in surf], al, dtype=npd, ref_pt=(0.25, 0.0, 0.0))
        got, g = sim.run(FlowData(al), ref_pt=(0.25, 0.0, 0.0), return_gamma=True)
        rg = np.concatenate([x.ravel() for x in ref["gamma"]]).astype(np.float64)
        if prec == 64:
            tol = 1e-8  # double path vs double oracle; the 20000-wide "infinite" panels cost ~1e-9
        else:
            tol = 2e-4  # float path vs float oracle (both carry ~1e-5 float error)
        scale = max(abs(float(ref["cl"])), 1e-3)
        assert abs(got.cl - float(ref["cl"])) <= tol * scale, (adeg, got.cl, ref["cl"])
        assert np.linalg.norm(g - rg) <= tol * max(np.linalg.norm(rg), 1e-6)
        assert abs(got.cd - float(ref["cdi"])) <= tol * max(abs(float(ref["cdi"])), 1e-6) + 1e-9
        cms = max(np.abs(ref["cm"]).max(), 1e-3)
        assert np.abs(np.array(got.cm) - ref["cm"]).max() <= tol * cms


def test_elliptic_lifting_line_kat(cuda):
    """tests/vlm_elliptic_coeffs.cpp:23-75: CL within 3% of 2 pi a/(1+2/AR)."""
    v = M.elliptic(20, 20).astype(np.float32)
    M.quarter_chord(v)
    sim = VLM("gb300", [v])
    a, b = 1.0, 5.0
    s = 0.5 * math.pi * a * b
    ar = (2 * b) ** 2 / s
    for adeg in (1, 2, 3, 4, 5, 10, 15):
        al = math.radians(adeg)
        cl = sim.run(FlowData(al)).cl
        ana = 2 * math.pi * al / (1 + 2 / ar)
        assert abs(cl - ana) / ana < 0.03, (adeg, cl, ana)


def test_square_two_surface_kat(cuda):
    """tests/vlm_square_coeffs.cpp:15-57 incl. the two-part split wing: CL within 1% of 2 pi a."""
    surfs = _cases()["split"]
    sim = VLM("gb300", surfs)
    for adeg in (1, 5, 10):
        al = math.radians(adeg)
        cl = sim.run(FlowData(al)).cl
        assert abs(cl - 2 * math.pi * al) / (2 * math.pi * al) < 0.01, (adeg, cl)
