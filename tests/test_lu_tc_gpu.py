"""Float LU of the library against LAPACK's float LU (sgetrf/sgetrs) on the
same matrices: the tensor-core trailing update (3xTF32, the default) must keep
the solution error at the level of a plain fp32 factorisation; the CUDA-core
path (GBVLM_LU_TC=0) likewise, and so must U12 = L11^-1 A12 formed as an
explicit inverse and a tensor-core product (the default) or by the
triangular solve (GBVLM_TC_TRSM=0); plain TF32 (GBVLM_LU_TC=1) only to TF32
accuracy.  Sizes cover one and several 128-column outer blocks, ragged
edges, panels split over a thread-block cluster, and a system taller than
4096 rows."""
import os

import numpy as np
import pytest
import torch
from scipy.linalg import lapack

from tinyvlm_gb300 import backend as B

pytestmark = pytest.mark.gpu


def _solve(A, b, mode, trsm="1"):
    old = os.environ.get("GBVLM_LU_TC")
    old_t = os.environ.get("GBVLM_TC_TRSM")
    os.environ["GBVLM_LU_TC"] = mode
    os.environ["GBVLM_TC_TRSM"] = trsm
    try:
        be = B.Backend(torch.float32)
        At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()  # column-major storage
        X = torch.from_numpy(np.ascontiguousarray(b)).cuda()
        lu = be.create_lu_solver()
        lu.init(At)
        lu.factorize(At)
        lu.solve(At, X)
        torch.cuda.synchronize()
        return X.cpu().numpy().astype(np.float64)
    finally:
        for k, v in (("GBVLM_LU_TC", old), ("GBVLM_TC_TRSM", old_t)):
            if v is None:
                del os.environ[k]
            else:
                os.environ[k] = v


def _matrix(n, seed, boost):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)).astype(np.float32)
    if boost:
        A += np.float32(boost * np.sqrt(n)) * np.eye(n, dtype=np.float32)
    b = rng.standard_normal((3, n)).astype(np.float32)
    return A, b


def _lapack_err(A, b, x_true):
    lu, piv, info = lapack.sgetrf(A)
    assert info == 0
    x, info = lapack.sgetrs(lu, piv, b.T)
    return np.abs(x.T.astype(np.float64) - x_true).max() / np.abs(x_true).max()


@pytest.mark.parametrize("n", [129, 256, 300, 1000, 1100, 2500, 4500])
@pytest.mark.parametrize("boost", [0.0, 2.0])
def test_lu_float_accuracy(cuda, n, boost):
    A, b = _matrix(n, 1000 + n, boost)
    x_true = np.linalg.solve(A.astype(np.float64), b.T.astype(np.float64)).T
    ref = _lapack_err(A, b, x_true)
    # tensor-core update with U12 through the explicit inverse of L11 (the
    # default) and through the triangular solve, and the CUDA-core path
    for mode, trsm in (("3", "1"), ("3", "0"), ("0", "1")):
        x = _solve(A, b, mode, trsm)
        err = np.abs(x - x_true).max() / np.abs(x_true).max()
        assert err <= 8.0 * ref + 1e-6, (mode, trsm, n, err, ref)


@pytest.mark.parametrize("n", [300, 1100])
def test_lu_tf32(cuda, n):
    A, b = _matrix(n, 2000 + n, 2.0)
    x_true = np.linalg.solve(A.astype(np.float64), b.T.astype(np.float64)).T
    x = _solve(A, b, "1")
    err = np.abs(x - x_true).max() / np.abs(x_true).max()
    assert err <= 5e-2, err  # tf32 operands: ~1e-3 relative per product


def test_batch_with_tall_system(cuda):
    """A 4608-unknown wing (8-CTA cluster panels for its first steps) in a
    batch with small ones: every solve within the batched path's bar of the double
    oracle."""
    from oracle import oracle as O
    from tinyvlm_gb300 import mesh as M
    from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts
    rng = np.random.default_rng(5)
    cases = []
    for nc, ns in [(48, 96), (8, 30), (4, 12)]:
        v = M.trapezoid(nc, ns, 8.0, 0.5, 15.0)
        M.quarter_chord(v)
        cases.append(M.Case(v.astype(np.float32), np.radians(rng.uniform(-6, 6, size=3)), {}))
    bs = BatchSolver(cases, mode="shared", refine=1)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=(0.25, 0.0, 0.0))
    bs.run()
    co, _ = bs.results()
    k = 0
    for c in cases:
        for r in O.vlm_shared([c.verts.astype(np.float64)], c.alphas, ref_pt=(0.25, 0.0, 0.0)):
            cl = float(r["cl"])
            assert abs(co[k, 0] - cl) <= 1e-5 * max(abs(cl), 1e-3), (c.n, k, co[k, 0], cl)
            k += 1
