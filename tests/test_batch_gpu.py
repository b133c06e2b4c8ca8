"""Batched steady solver (C ABI gbvlm_batch_*) against the double oracle.

Target of the batched mixed-precision path: CL, CM and CDi within a relative
1e-5 of the full double solve (geometry, assembly and LU in double).  Also
checks the result of every case is the same alone and inside the batch."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts
from tinyvlm_gb300.vlm import VLM, FlowData

pytestmark = pytest.mark.gpu
REF = (0.25, 0.0, 0.0)
TOL = 1e-5


def _ref(mode, c):
    v64 = c.verts.astype(np.float64)
    if mode == "shared":
        return O.vlm_shared([v64], c.alphas, ref_pt=REF)
    return [O.vlm_run([v64], a, dtype=np.float64, ref_pt=REF) for a in c.alphas]


def _check(co, gam, cases, mode):
    k = 0
    cl_all = [float(r["cl"]) for c in cases for r in _ref(mode, c)]
    guard = 1e-3 * max(abs(x) for x in cl_all)
    for c in cases:
        for r in _ref(mode, c):
            cl = float(r["cl"])
            assert abs(co[k, 0] - cl) <= TOL * max(abs(cl), guard), ("CL", mode, k, co[k, 0], cl)
            cms = max(np.abs(r["cm"]).max(), 1e-6)
            assert np.abs(co[k, 2:5] - r["cm"]).max() <= TOL * cms, ("CM", mode, k, co[k, 2:5], r["cm"])
            cd = float(r["cdi"])
            assert abs(co[k, 1] - cd) <= TOL * max(abs(cd), 1e-6) + 1e-12, ("CDi", mode, k, co[k, 1], cd)
            if gam is not None:
                g = np.concatenate([x.ravel() for x in r["gamma"]])
                assert np.linalg.norm(gam[k] - g) <= 1e-5 * np.linalg.norm(g) + 1e-7, ("gamma", mode, k)
            k += 1


@pytest.mark.parametrize("mode", ["shared", "exact"])
@pytest.mark.parametrize("refine", [0, 1])
def test_batch_matches_double_oracle(cuda, mode, refine):
    cases = M.batch_cases(10, seed=11, n_alpha=3, nc_range=(4, 12), ns_range=(4, 24))
    bs = BatchSolver(cases, mode=mode, refine=refine)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run(want_gamma=True)
    co, gam = bs.results(gamma=True)
    _check(co, gam, cases, mode)
    # run again (graph replay) with new angles
    for c in cases:
        c.alphas = c.alphas[::-1].copy()
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run(want_gamma=False)
    co2, _ = bs.results()
    _check(co2, None, cases, mode)


@pytest.mark.parametrize("mode", ["shared", "exact"])
def test_fp64_residual_converges_to_the_double_solution(cuda, mode):
    """GBVLM_BATCH_FP64_RESIDUAL: the residual's AIC is the stored float AIC plus its float-pair correction, so
    the refinement converges to the double system's solution.  Two sweeps bring every gamma within 3e-7 of
    ||gamma_64|| (the float rounding of the stored result is 6e-8) and CL/CM within 5e-7 (the loads form their
    force and moment terms in float and sum them in double; 1e-7 in the shared formulation).  Cases in all three
    LU size groups (n > 1024, 384 < n <= 1024, n <= 384), each group's correction on its own graph branch;
    the graph, its replay, the eager launch sequence and the staged (profiled) run agree."""
    cases = M.batch_cases(12, seed=17, n_alpha=2, nc_range=(4, 32), ns_range=(4, 64))
    n = [c.n for c in cases]
    assert max(n) > 1024 and min(n) <= 384 and any(384 < x <= 1024 for x in n)
    bs = BatchSolver(cases, mode=mode, refine=2, fp64_residual=True)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run(want_gamma=True)
    co, gam = bs.results(gamma=True)
    k = 0
    for c in cases:
        for r in _ref(mode, c):
            g = np.concatenate([x.ravel() for x in r["gamma"]])
            assert np.linalg.norm(gam[k] - g) <= 3e-7 * np.linalg.norm(g), ("gamma", mode, k)
            cl = float(r["cl"])
            assert abs(co[k, 0] - cl) <= 5e-7 * max(abs(cl), 1e-3), ("CL", mode, k, co[k, 0], cl)
            assert np.abs(co[k, 2:5] - r["cm"]).max() <= 5e-7 * max(np.abs(r["cm"]).max(), 1e-6), ("CM", mode, k)
            k += 1
    bs.run(want_gamma=True)  # replay
    co2, gam2 = bs.results(gamma=True)
    np.testing.assert_array_equal(co2, co)
    for a, b in zip(gam2, gam):
        np.testing.assert_array_equal(a, b)
    bs.run(want_gamma=True, graph=False)
    co3, _ = bs.results(gamma=True)
    np.testing.assert_allclose(co3, co, rtol=1e-12, atol=1e-15)
    bs.profile()
    co4, _ = bs.results()
    np.testing.assert_allclose(co4, co, rtol=1e-12, atol=1e-15)


def test_fp64_residual_needs_a_refinement_sweep(cuda):
    from tinyvlm_gb300._lib import GbvlmError
    cases = M.batch_cases(2, seed=1, n_alpha=1, nc_range=(4, 6), ns_range=(4, 6))
    with pytest.raises(GbvlmError, match="GBVLM_ERR_ARG"):
        BatchSolver(cases, mode="shared", refine=0, fp64_residual=True)


def test_non_finite_input_is_reported(cuda):
    """A case whose vertices hold a NaN is reported by gbvlm_batch_results (GBVLM_ERR_ARG naming the case), the
    next set_inputs/run with clean vertices is valid again, and a non-finite angle is refused at set_inputs."""
    from tinyvlm_gb300._lib import GbvlmError
    cases = M.batch_cases(4, seed=2, n_alpha=2, nc_range=(4, 6), ns_range=(4, 8))
    bs = BatchSolver(cases, mode="shared", refine=1)
    v = pack_verts(cases).copy()
    v[sum(4 * (c.ns + 1) * (c.nc + 1) for c in cases[:2])] = np.nan  # x of case 2's first vertex
    bs.set_inputs(v, pack_alphas(cases), ref_pt=REF)
    bs.run()
    with pytest.raises(GbvlmError, match="case 2: non-finite"):
        bs.results()
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run()
    co, _ = bs.results()
    _check(co, None, cases, "shared")
    al = pack_alphas(cases).copy()
    al[3] = np.inf
    with pytest.raises(GbvlmError, match="GBVLM_ERR_ARG"):
        bs.set_inputs(pack_verts(cases), al, ref_pt=REF)


def test_batch_large_cases(cuda):
    """Sizes up to the full workload's largest (32 x 64 = 2048 panels)."""
    cases = M.batch_cases(4, seed=3, n_alpha=2, nc_range=(28, 32), ns_range=(56, 64))
    bs = BatchSolver(cases, mode="shared", refine=1)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run()
    co, _ = bs.results()
    _check(co, None, cases, "shared")


def test_alone_equals_in_mix(cuda):
    cases = M.batch_cases(8, seed=5, n_alpha=2, nc_range=(4, 10), ns_range=(4, 20))
    bs = BatchSolver(cases, mode="exact", refine=1)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run()
    mix, _ = bs.results()
    for i, c in enumerate(cases):
        one = BatchSolver([c], mode="exact", refine=1)
        one.set_inputs(pack_verts([c]), pack_alphas([c]), ref_pt=REF)
        one.run()
        alone, _ = one.results()
        np.testing.assert_allclose(alone, mix[2 * i:2 * i + 2], rtol=1e-12, atol=1e-14)


def test_batch_vs_plain_double_path(cuda):
    """The batched mixed-precision path against the plain per-solve double GPU path."""
    cases = M.batch_cases(3, seed=9, n_alpha=2, nc_range=(6, 10), ns_range=(8, 16))
    bs = BatchSolver(cases, mode="exact", refine=1)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run()
    co, _ = bs.results()
    k = 0
    for c in cases:
        plain = VLM("gb300", [c.verts], precision=64)
        for a in c.alphas:
            r = plain.run(FlowData(a), ref_pt=REF)
            assert abs(co[k, 0] - r.cl) <= TOL * max(abs(r.cl), 1e-3), (co[k, 0], r.cl)
            k += 1


def test_eager_equals_graph_across_size_groups(cuda):
    """Systems from all three LU size groups (n > 1024, 384 < n <= 1024,
    n <= 384, factored on separate graph branches): the captured graph and
    the kernel-by-kernel launch give identical results, and a large system
    alone equals the same system inside the mixed batch."""
    big = M.batch_cases(2, seed=11, n_alpha=2, nc_range=(28, 32), ns_range=(48, 64))
    mid = M.batch_cases(3, seed=12, n_alpha=2, nc_range=(16, 20), ns_range=(30, 40))
    small = M.batch_cases(4, seed=13, n_alpha=2, nc_range=(4, 8), ns_range=(4, 20))
    cases = big + mid + small
    assert max(c.n for c in cases) > 1024 and min(c.n for c in cases) <= 384
    bs = BatchSolver(cases, mode="shared", refine=0)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run()
    graph, _ = bs.results()
    bs.run(graph=False)
    eager, _ = bs.results()
    np.testing.assert_array_equal(graph, eager)
    one = BatchSolver([big[0]], mode="shared", refine=0)
    one.set_inputs(pack_verts([big[0]]), pack_alphas([big[0]]), ref_pt=REF)
    one.run(graph=False)
    alone, _ = one.results()
    np.testing.assert_allclose(alone, graph[0:2], rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("depth", [1, 2, 3])
def test_pipeline_equals_single_solver(cuda, depth):
    """BatchPipeline: batches with different angles submitted back to back, up to `depth` in flight, each
    collected first in first out; every batch's coefficients and circulations are bitwise those of one
    BatchSolver run on the same inputs.  Then the device-resident run() path on every slot in turn."""
    cases = M.batch_cases(24, seed=11, n_alpha=3, nc_range=(4, 24), ns_range=(4, 48))
    from tinyvlm_gb300.batch import BatchPipeline
    rng = np.random.default_rng(5)
    batches = [np.deg2rad(rng.uniform(-8, 8, len(pack_alphas(cases)))) for _ in range(7)]
    single = BatchSolver(cases, mode="shared", refine=1)
    want = []
    for al in batches:
        single.set_inputs(pack_verts(cases), al, ref_pt=REF)
        single.run(want_gamma=True)
        co, g = single.results(gamma=True)
        want.append((co, np.concatenate(g)))
    pipe = BatchPipeline(cases, depth=depth, mode="shared", refine=1)
    got, tickets = {}, []
    for al in batches:
        if pipe.full():
            g = np.zeros(pipe.gamma_floats, np.float32)
            t, co, _ = pipe.collect(g=g)
            got[t] = (co, g)
        tickets.append(pipe.submit(pack_verts(cases), al, ref_pt=REF, want_gamma=True))
        assert pipe.pending() <= depth
    while pipe.pending():
        g = np.zeros(pipe.gamma_floats, np.float32)
        t, co, _ = pipe.collect(g=g)
        got[t] = (co, g)
    assert sorted(got) == tickets == list(range(len(batches)))
    for t, (co, g) in got.items():
        np.testing.assert_array_equal(co, want[t][0])
        np.testing.assert_array_equal(g, want[t][1])
    # resident inputs: each slot solves the last batch again
    pipe.set_inputs(pack_verts(cases), batches[-1], ref_pt=REF)
    slots = [pipe.run() for _ in range(2 * depth)]
    assert slots == [(i + len(batches)) % depth for i in range(2 * depth)]
    for s, st in zip(pipe.slots, pipe.streams):
        co, _ = s.results(stream=st)
        np.testing.assert_array_equal(co, want[-1][0])


def test_pipeline_refusals(cuda):
    cases = M.batch_cases(3, seed=12, n_alpha=2, nc_range=(4, 6), ns_range=(4, 8))
    from tinyvlm_gb300.batch import BatchPipeline
    pipe = BatchPipeline(cases, depth=2)
    with pytest.raises(RuntimeError, match="no batch in flight"):
        pipe.collect()
    pipe.submit(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    with pytest.raises(ValueError, match="without want_gamma"):
        pipe.collect(g=np.zeros(pipe.gamma_floats, np.float32))
    pipe.submit(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    with pytest.raises(RuntimeError, match="collect one first"):
        pipe.submit(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    with pytest.raises(RuntimeError, match="in flight first"):
        pipe.run()
    assert [pipe.collect()[0] for _ in range(2)] == [0, 1]
    with pytest.raises(ValueError):
        BatchPipeline(cases, depth=0)


@pytest.mark.parametrize("mode", ["shared", "exact"])
@pytest.mark.parametrize("rows", [1, 2, 3, 4])
def test_assembly_rows_per_tile(cuda, rows, mode):
    """Float assembly tiles of 1-4 chordwise ring rows (batch.assembly_rows; k_batch_assemble_rows beyond one):
    the batch matches the double oracle, CDi included.  The cases include ring-row counts that are not multiples
    of the rows per tile (the trailing-edge row, with its wake rings, in a shorter last tile) and spans wider
    than one 128-ring chunk: up to 150 spanwise panels, whose narrow wake panels 50 chords from the wing are
    where the Trefftz influence needs the wake's own frame (exact mode, the wake tilted by alpha).  With the
    FP64 residual (whose correction kernel keeps one-row tiles and reads the float AIC these tiles write) the
    circulations still converge to the double solution."""
    from tinyvlm_gb300 import autotune as A
    cases = M.batch_cases(8, seed=21, n_alpha=2, nc_range=(4, 11), ns_range=(4, 150))
    assert (rows == 1 or any(c.nc % rows for c in cases)) and max(c.ns for c in cases) > 128
    saved = A.current()
    try:
        A.set_params({"batch.assembly_rows": rows})
        bs = BatchSolver(cases, mode=mode, refine=1, tuned=False)
        bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
        bs.run(want_gamma=True)
        co, gam = bs.results(gamma=True)
        _check(co, gam, cases, mode)
        bf = BatchSolver(cases, mode=mode, refine=2, fp64_residual=True, tuned=False)
        bf.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
        bf.run(want_gamma=True)
        _, gam64 = bf.results(gamma=True)
    finally:
        A.set_params(saved)
    k = 0
    for c in cases:
        for r in _ref(mode, c):
            g = np.concatenate([x.ravel() for x in r["gamma"]])
            assert np.linalg.norm(gam64[k] - g) <= 3e-7 * np.linalg.norm(g), ("gamma fp64 residual", mode, rows, k)
            k += 1


def test_four_size_groups(cuda):
    """batch.group_mid: a fourth LU size group (n > 1024, 640 < n <= 1024, 256 < n <= 640, n <= 256), each on its
    own graph branch: the batch matches the double oracle, the graph equals the kernel-by-kernel launch and its
    replay, and the same batch in three groups gives the same coefficients to float rounding."""
    from tinyvlm_gb300 import autotune as A
    big = M.batch_cases(2, seed=31, n_alpha=2, nc_range=(28, 32), ns_range=(48, 64))
    upper = M.batch_cases(2, seed=32, n_alpha=2, nc_range=(20, 24), ns_range=(36, 42))
    lower = M.batch_cases(2, seed=33, n_alpha=2, nc_range=(12, 16), ns_range=(24, 36))
    small = M.batch_cases(3, seed=34, n_alpha=2, nc_range=(4, 8), ns_range=(4, 24))
    cases = big + upper + lower + small
    n = sorted(c.n for c in cases)
    assert n[-1] > 1024 and any(640 < x <= 1024 for x in n) and any(256 < x <= 640 for x in n) and n[0] <= 256
    saved = A.current()
    try:
        A.set_params({"batch.group_hi": 1024, "batch.group_mid": 640, "batch.group_lo": 256})
        bs = BatchSolver(cases, mode="shared", refine=1, tuned=False)
        bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
        bs.run(want_gamma=True)
        co, gam = bs.results(gamma=True)
        bs.run(want_gamma=True)
        co_r, _ = bs.results()
        bs.run(graph=False)
        co_e, _ = bs.results()
        A.set_params({"batch.group_mid": 0})
        b3 = BatchSolver(cases, mode="shared", refine=1, tuned=False)
        b3.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
        b3.run()
        co3, _ = b3.results()
        from tinyvlm_gb300._lib import GbvlmError
        A.set_params({"batch.group_mid": 2048})
        with pytest.raises(GbvlmError, match="group_mid"):
            BatchSolver(cases, mode="shared", refine=1, tuned=False)
    finally:
        A.set_params(saved)
    _check(co, gam, cases, "shared")
    np.testing.assert_array_equal(co_r, co)
    np.testing.assert_array_equal(co_e, co)
    np.testing.assert_allclose(co3, co, rtol=1e-12, atol=1e-14)
