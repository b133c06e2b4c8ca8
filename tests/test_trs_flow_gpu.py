"""Dataflow triangular solves of the batched solver (k_trs_flow: one
persistent launch, 128-row blocks of every system and every group of 8
right-hand sides handed out in dependency order) against the per-system
solves (GBVLM_TRS_FLOW=0) and the double oracle.

Sizes sit on both sides of the 128-row block edges (last blocks of 1, 127
and 128 rows, single-block systems, 10 blocks) and 11 angles make two
groups of right-hand sides, the second with 3.  A single system of 4560
unknowns with 20 angles (three groups) runs against the blocked
tensor-core solve it replaced."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts

pytestmark = pytest.mark.gpu
REF = (0.25, 0.0, 0.0)
SHAPES = [(32, 40), (16, 16), (3, 43), (1, 127), (8, 16), (10, 30), (4, 100), (2, 5), (1, 1)]


def _cases(n_alpha, seed=7):
    rng = np.random.default_rng(seed)
    out = []
    for nc, ns in SHAPES:
        v = M.trapezoid(nc, ns, float(rng.uniform(4, 12)), float(rng.uniform(0.3, 1.0)), float(rng.uniform(0, 35)))
        M.quarter_chord(v)
        al = np.radians(rng.uniform(-8, 8, size=n_alpha))
        out.append(M.Case(v.astype(np.float32), al, dict(nc=nc, ns=ns)))
    return out


def _solve(cases, flow, refine, mode="shared"):
    old = os.environ.get("GBVLM_TRS_FLOW")
    os.environ["GBVLM_TRS_FLOW"] = "1" if flow else "0"
    try:
        bs = BatchSolver(cases, mode=mode, refine=refine)
    finally:
        if old is None:
            del os.environ["GBVLM_TRS_FLOW"]
        else:
            os.environ["GBVLM_TRS_FLOW"] = old
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run(want_gamma=True)
    return bs.results(gamma=True)


@pytest.mark.parametrize("mode", ["shared", "exact"])
def test_flow_equals_per_system_solve(cuda, mode):
    cases = _cases(11 if mode == "shared" else 2)
    assert sorted(c.n for c in cases)[:3] == [1, 10, 127] and max(c.n for c in cases) == 1280
    co_f, g_f = _solve(cases, True, 0, mode)
    co_s, g_s = _solve(cases, False, 0, mode)
    # same float factorisation, float solves summed in another order
    for a, b in zip(g_f, g_s):
        assert np.linalg.norm(a - b) <= 2e-5 * np.linalg.norm(b) + 1e-7
    np.testing.assert_allclose(co_f[:, 0], co_s[:, 0], rtol=2e-5, atol=1e-7)


def test_flow_refined_matches_double_oracle(cuda):
    cases = _cases(11, seed=8)
    co, gam = _solve(cases, True, 1)
    k = 0
    for c in cases:
        for r in O.vlm_shared([c.verts.astype(np.float64)], c.alphas, ref_pt=REF):
            cl = float(r["cl"])
            assert abs(co[k, 0] - cl) <= 1e-5 * max(abs(cl), 1e-3), (c.n, k, co[k, 0], cl)
            g = np.concatenate([x.ravel() for x in r["gamma"]])
            assert np.linalg.norm(gam[k] - g) <= 1e-5 * np.linalg.norm(g) + 1e-7, (c.n, k)
            k += 1


def test_flow_replay_is_deterministic(cuda):
    """Items go to whichever CTA takes them, but each block's sums run in a
    fixed order: replays give identical bits."""
    cases = _cases(8, seed=9)
    bs = BatchSolver(cases, mode="shared", refine=1)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run()
    a, _ = bs.results()
    for _ in range(3):
        bs.run()
        b, _ = bs.results()
        np.testing.assert_array_equal(a, b)


def test_flow_single_large_system_groups(cuda):
    rng = np.random.default_rng(11)
    v = M.trapezoid(24, 190, 9.0, 0.6, 20.0)
    M.quarter_chord(v)
    cases = [M.Case(v.astype(np.float32), np.radians(rng.uniform(-8, 8, size=20)), {})]
    assert cases[0].n == 4560
    co_f, g_f = _solve(cases, True, 1)
    co_s, g_s = _solve(cases, False, 1)
    for a, b in zip(g_f, g_s):
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b) + 1e-7
    np.testing.assert_allclose(co_f[:, 0], co_s[:, 0], rtol=1e-5, atol=1e-7)
