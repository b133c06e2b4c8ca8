"""Pin the oracle to the reference's own known-answer tests (CPU only).

The reference stores no golden arrays; its tests pin this path analytically:
  * tests/vlm_elliptic_coeffs.cpp:23-75  elliptic wing, CL within 3 % of
    lifting-line 2 pi alpha / (1 + 2/AR), alpha in {0,1,2,3,4,5,10,15} deg;
  * tests/vlm_square_coeffs.cpp:15-57    "infinite" rectangles (semispan
    40000) incl. a two-surface split, CL within 1 % of 2 pi alpha.
The reference meshes come from tests/golden/ref_meshes.npz (the numbers
the reference's own plot3d reader returns for its mesh files, written by
tests/golden/make_ref_golden.py); the generated equivalents run too.
Golden fixtures made by tests/golden/make_golden.py are re-checked here so a
change to the oracle is caught.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests import ref_fixtures as R
from tinyvlm_gb300 import mesh as M

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ALPHAS = [0, 1, 2, 3, 4, 5, 10, 15]


def _elliptic_ar(a=1.0, b=5.0):
    return (2 * b) ** 2 / (0.5 * math.pi * a * b)


def _check_elliptic(v, tol=0.03):
    ar = _elliptic_ar()
    for adeg in ALPHAS:
        al = np.float32(math.radians(adeg))
        cl = O.vlm_run([v], al)["cl"]
        ana = 2 * math.pi * float(al) / (1 + 2 / ar)
        err = 0.0 if ana < 1.19209e-07 else abs(cl - ana) / ana
        assert err <= tol, (adeg, cl, ana)


def _check_square(surfs, tol=0.01):
    for adeg in ALPHAS:
        al = np.float32(math.radians(adeg))
        cl = O.vlm_run(surfs, al)["cl"]
        ana = 2 * math.pi * float(al)
        err = 0.0 if ana < 1.19209e-07 else abs(cl - ana) / ana
        assert err <= tol, (adeg, cl, ana)


def test_elliptic_kat_generated():
    v = M.elliptic(30, 30).astype(np.float32)
    M.quarter_chord(v)
    _check_elliptic(v)


def test_square_kat_generated():
    for ns, nc in ((2, 4), (10, 5), (20, 5)):
        v = M.rectangular(nc, ns, 1.0, 40000.0).astype(np.float32)
        M.quarter_chord(v)
        _check_square([v])
    a = M.rectangular(2, 2, 1.0, 20000.0, 0.0).astype(np.float32)
    b = M.rectangular(2, 2, 1.0, 20000.0, 20000.0).astype(np.float32)
    M.quarter_chord(a)
    M.quarter_chord(b)
    _check_square([a, b])


def test_elliptic_kat_reference_mesh():
    _check_elliptic(R.mesh("elliptic_45x45"))


def test_square_kat_reference_meshes():
    _check_square([R.mesh("infinite_rectangular_2x2_part0"), R.mesh("infinite_rectangular_2x2_part1")])
    for m in ("infinite_rectangular_2x4", "infinite_rectangular_10x5", "infinite_rectangular_20x5"):
        _check_square([R.mesh(m)])


def test_generated_square_equals_reference_mesh():
    ref = R.mesh("infinite_rectangular_10x5")
    v = M.rectangular(10, 5, 1.0, 40000.0).astype(np.float32)
    M.quarter_chord(v)
    np.testing.assert_allclose(v, ref, rtol=1e-6, atol=1e-6)


def test_float_and_double_agree():
    v = M.trapezoid(6, 12, 8.0, 0.5, 20.0).astype(np.float32)
    M.quarter_chord(v)
    al = math.radians(4.0)
    r32 = O.vlm_run([v], al)
    r64 = O.vlm_run([v.astype(np.float64)], al, dtype=np.float64)
    assert abs(r32["cl"] - r64["cl"]) / abs(r64["cl"]) < 2e-4


def test_trefftz_cdi_close_to_elliptic_theory():
    """Loose analytical check CDi ~ CL^2/(pi AR) (vlm_elliptic_coeffs.cpp:27-29)."""
    v = M.elliptic(16, 24).astype(np.float64)
    M.quarter_chord(v)
    r = O.vlm_run([v], math.radians(5.0), dtype=np.float64)
    ana = r["cl"] ** 2 / (math.pi * _elliptic_ar())
    assert abs(r["cdi"] - ana) / ana < 0.05


@pytest.mark.parametrize("name", ["vlm_generated.json", "vlm_reference_meshes.json"])
def test_golden_fixtures(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    from tests.golden.make_golden import build_case
    with open(path) as f:
        data = json.load(f)
    for case in data["cases"]:
        surfs = build_case(case)
        if surfs is None:
            continue
        dt = np.float32 if case["precision"] == 32 else np.float64
        r = O.vlm_run([s.astype(dt) for s in surfs], case["alpha"], dtype=dt, ref_pt=case["ref_pt"])
        tol = 1e-6 if dt == np.float32 else 1e-12
        assert abs(r["cl"] - case["cl"]) <= tol * max(abs(case["cl"]), 1e-3), case["name"]
        assert abs(r["cdi"] - case["cdi"]) <= tol * max(abs(case["cdi"]), 1e-6) + 1e-12, case["name"]
        np.testing.assert_allclose(r["cm"], case["cm"], rtol=tol, atol=tol * 1e-2)
