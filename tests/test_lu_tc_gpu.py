"""Float LU of the library against LAPACK's float LU (sgetrf/sgetrs) on the
same matrices: the tensor-core trailing update (3xTF32, the default) must keep
the solution error at the level of a plain fp32 factorisation; the CUDA-core
path (GBVLM_LU_TC=0) likewise; plain TF32 (GBVLM_LU_TC=1) only to TF32
accuracy.  Sizes cover one and several 128-column outer blocks, ragged
edges, and panels split over a thread-block cluster."""
import os

import numpy as np
import pytest
import torch
from scipy.linalg import lapack

from tinyvlm_gb300 import backend as B

pytestmark = pytest.mark.gpu


def _solve(A, b, mode):
    old = os.environ.get("GBVLM_LU_TC")
    os.environ["GBVLM_LU_TC"] = mode
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
        if old is None:
            del os.environ["GBVLM_LU_TC"]
        else:
            os.environ["GBVLM_LU_TC"] = old


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


@pytest.mark.parametrize("n", [129, 256, 300, 1000, 1100, 2500])
@pytest.mark.parametrize("boost", [0.0, 2.0])
def test_lu_float_accuracy(cuda, n, boost):
    A, b = _matrix(n, 1000 + n, boost)
    x_true = np.linalg.solve(A.astype(np.float64), b.T.astype(np.float64)).T
    ref = _lapack_err(A, b, x_true)
    for mode in ("3", "0"):
        x = _solve(A, b, mode)
        err = np.abs(x - x_true).max() / np.abs(x_true).max()
        assert err <= 8.0 * ref + 1e-6, (mode, n, err, ref)


@pytest.mark.parametrize("n", [300, 1100])
def test_lu_tf32(cuda, n):
    A, b = _matrix(n, 2000 + n, 2.0)
    x_true = np.linalg.solve(A.astype(np.float64), b.T.astype(np.float64)).T
    x = _solve(A, b, "1")
    err = np.abs(x - x_true).max() / np.abs(x_true).max()
    assert err <= 5e-2, err  # tf32 operands: ~1e-3 relative per product
