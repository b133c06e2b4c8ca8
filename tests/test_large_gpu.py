"""Large steady path: one AIC, many right-hand sides (the 64-alpha sweep of
the 16,384-panel workload), against the full double solve at 1e-5: on a
24 x 32 elliptic wing with and without refinement, and at the configured
128 x 128 size on the reference's own elliptic wing.

The literal analytic planform, chord sqrt(1 - (2y/b)^2) down to a zero tip
chord with cosine spanwise spacing, is not used at the large size.  Its
degenerate tip rings make the AIC singular to working precision as the
spanwise count grows (cond_1 4.6e6 at 64 x 64, 1.5e13 at 80 x 80), beyond
any solve that stores the AIC in float.  The reference's elliptic meshes
end at a 0.0707 tip chord (cond_1 1.6e3 at 16 x 16, 6.4e3 at 45 x 45)."""
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


def _errors(co, gam, ref):
    """Per-alpha errors against the double solve: guarded CL and CM, relative gamma norm."""
    cls = np.array([float(r["cl"]) for r in ref])
    guard = 1e-3 * np.abs(cls).max()
    cms = np.array([np.asarray(r["cm"], np.float64) for r in ref])
    cm_guard = 1e-3 * np.abs(cms[:, 1]).max()
    e_cl, e_cm, e_g = [], [], []
    for k, r in enumerate(ref):
        e_cl.append(abs(co[k, 0] - cls[k]) / max(abs(cls[k]), guard))
        e_cm.append(abs(co[k, 3] - cms[k, 1]) / max(abs(cms[k, 1]), cm_guard))
        g = np.concatenate([x.ravel() for x in r["gamma"]])
        e_g.append(np.linalg.norm(gam[k] - g) / np.linalg.norm(g))
    return np.array(e_cl), np.array(e_cm), np.array(e_g)


def test_config_c_16384_panels_64_alphas_vs_full_double(cuda):
    """Config C at its configured size: the reference's elliptic 128 x 128 = 16,384-panel wing
    (mesh/elliptic_128x128.x), 64 alphas in [-10, 10] deg on one AIC; float AIC, tensor-core LU and one
    refinement sweep with the FP64 residual (float AIC plus its float-pair correction) against the oracle's
    full double solve (double assembly, LAPACK
    dgetrf/dgetrs).  Every alpha: CL and CM_y (guarded near zero lift) and ||gamma - gamma_64|| /
    ||gamma_64|| within 1e-5."""
    from tests import ref_fixtures as R
    v = R.mesh("elliptic_128x128")
    al = np.radians(np.linspace(-10.0, 10.0, 64))
    case = M.Case(v, al, {})
    bs = BatchSolver([case], mode="shared", refine=1, fp64_residual=True)
    bs.set_inputs(pack_verts([case]), pack_alphas([case]))
    bs.run(want_gamma=True)
    co, gam = bs.results(gamma=True)
    ref = O.vlm_shared([v.astype(np.float64)], al)
    e_cl, e_cm, e_g = _errors(co, gam, ref)
    print("config C max errors: CL %.2e CM %.2e gamma %.2e" % (e_cl.max(), e_cm.max(), e_g.max()))
    assert e_cl.max() <= 1e-5 and e_cm.max() <= 1e-5 and e_g.max() <= 1e-5


@pytest.mark.parametrize("prec,tol", [(64, 1e-9), (32, 2e-4)])
def test_plain_shared_sweep_matches_oracle(cuda, prec, tol):
    """VLM.run_shared (gbvlm_vlm_run_shared): the plain per-operator path of the shared-AIC sweep, double and
    float, against the oracle's sweep."""
    from tinyvlm_gb300.vlm import VLM
    v = M.elliptic(12, 16).astype(np.float32)
    M.quarter_chord(v)
    al = np.radians(np.linspace(-10.0, 10.0, 9))
    res, gam = VLM("gb300", [v], precision=prec).run_shared(al, ref_pt=(0.25, 0.0, 0.0), return_gamma=True)
    npd = np.float64 if prec == 64 else np.float32
    ref = O.vlm_shared([v.astype(npd)], al, dtype=npd, ref_pt=(0.25, 0.0, 0.0))
    guard = 1e-3 * max(abs(float(r["cl"])) for r in ref)
    for k, (r, o) in enumerate(zip(ref, res)):
        assert abs(o.cl - float(r["cl"])) <= tol * max(abs(float(r["cl"])), guard), (k, o.cl, float(r["cl"]))
        np.testing.assert_allclose(o.cm, np.asarray(r["cm"], np.float64), rtol=tol * 10, atol=tol * 1e-2)
        g = np.concatenate([x.ravel() for x in r["gamma"]]).astype(np.float64)
        assert np.linalg.norm(gam[k] - g) <= tol * 10 * np.linalg.norm(g)
