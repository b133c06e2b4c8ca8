"""The rest of the vlm::Backend contract through the C ABI, on device arrays
of the library's own memory manager (no PyTorch): Memory (alloc, strided
copy, fill), BLAS (gemv, gemm, axpy 1-D / 2-D, scal, norm), LSQ (least
squares, LAPACK ?gels semantics), the strided 2-D sum, streams and events.
References are numpy in double."""
import ctypes

import numpy as np
import pytest

from tinyvlm_gb300 import backend as B
from tinyvlm_gb300 import device as D
from tinyvlm_gb300._lib import GbvlmError

pytestmark = pytest.mark.gpu

PREC = [(np.float32, 2e-6), (np.float64, 1e-13)]


def _dev(x):
    return D.DeviceArray.from_numpy(x)


def test_memory_roundtrip_fill_and_strided_copy(cuda):
    be = B.Backend(np.float64)
    mem = be.create_memory_manager()
    x = np.arange(24, dtype=np.float64)
    p = mem.alloc(mem.DEVICE, x.nbytes)
    h = mem.alloc(mem.HOST, x.nbytes)
    try:
        mem.copy(mem.DEVICE, p, 1, mem.HOST, x.ctypes.data, 1, 8, 24)
        out = np.zeros(24)
        mem.copy(mem.HOST, out.ctypes.data, 1, mem.DEVICE, p, 1, 8, 24)
        np.testing.assert_array_equal(out, x)
        # strided: every third element into a packed host buffer (a column of a (8, 3) view)
        col = np.zeros(8)
        mem.copy(mem.HOST, col.ctypes.data, 1, mem.DEVICE, p + 8, 3, 8, 8)
        np.testing.assert_array_equal(col, x[1::3])
        mem.fill(mem.DEVICE, p + 16, 3, -2.5, 8)
        mem.copy(mem.HOST, out.ctypes.data, 1, mem.DEVICE, p, 1, 8, 24)
        want = x.copy()
        want[2::3] = -2.5
        np.testing.assert_array_equal(out, want)
        # pinned host memory is usable as a host buffer
        mem.copy(mem.HOST, h, 1, mem.DEVICE, p, 1, 8, 24)
        got = np.frombuffer((ctypes.c_double * 24).from_address(h), np.float64)
        np.testing.assert_array_equal(got, want)
    finally:
        mem.free(mem.DEVICE, p)
        mem.free(mem.HOST, h)


def test_device_array_stream_and_events(cuda):
    s = D.Stream()
    x = np.random.default_rng(0).standard_normal((5, 7)).astype(np.float32)
    a = D.DeviceArray.from_numpy(x, stream=s)
    b = D.DeviceArray.zeros((5, 7), np.float32, stream=s)
    e0, e1 = D.Event(), D.Event()
    e0.record(s)
    b.copy_from(a, stream=s)
    e1.record(s)
    s.synchronize()
    assert e0.elapsed_time(e1) >= 0.0
    np.testing.assert_array_equal(b.numpy(), x)
    sm, free, total = D.device_info()
    assert sm >= 1 and 0 < free <= total


@pytest.mark.parametrize("npd,tol", PREC)
@pytest.mark.parametrize("trans", [0, 1])
def test_gemv(cuda, npd, tol, trans):
    rng = np.random.default_rng(1)
    m, n = 37, 23
    A = rng.standard_normal((m, n))
    x = rng.standard_normal(m if trans else n)
    y0 = rng.standard_normal(n if trans else m)
    be = B.Backend(npd)
    dA, dx, dy = _dev(np.ascontiguousarray(A.T).astype(npd)), _dev(x.astype(npd)), _dev(y0.astype(npd))
    be.blas.gemv(0.7, dA, dx, -1.3, dy, trans)
    op = A.T if trans else A
    want = 0.7 * op.astype(npd).astype(np.float64) @ x.astype(npd) - 1.3 * y0.astype(npd)
    np.testing.assert_allclose(dy.numpy(), want, rtol=tol * 10, atol=tol * 10 * np.abs(want).max())


@pytest.mark.parametrize("npd,tol", PREC)
@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_gemm(cuda, npd, tol, ta, tb):
    rng = np.random.default_rng(2)
    m, n, k = 70, 45, 33
    opA = rng.standard_normal((m, k))
    opB = rng.standard_normal((k, n))
    A = opA.T if ta else opA  # stored matrix
    Bm = opB.T if tb else opB
    C0 = rng.standard_normal((m, n))
    be = B.Backend(npd)
    # a C-ordered (cols, rows) array holds the column-major matrix
    dA, dB, dC = [_dev(np.ascontiguousarray(X.T).astype(npd)) for X in (A, Bm, C0)]
    be.blas.gemm(1.5, dA, dB, 0.5, dC, ta, tb)
    want = 1.5 * opA.astype(npd).astype(np.float64) @ opB.astype(npd) + 0.5 * C0.astype(npd)
    got = dC.numpy().T
    np.testing.assert_allclose(got, want, rtol=tol * 40, atol=tol * 40 * np.abs(want).max())
    # beta = 0 does not read C (BLAS semantics): NaN in C must not leak
    dC.fill(np.nan)
    be.blas.gemm(1.0, dA, dB, 0.0, dC, ta, tb)
    assert np.isfinite(dC.numpy()).all()


@pytest.mark.parametrize("npd,tol", PREC)
def test_axpy_scal_norm_and_2d_axpy(cuda, npd, tol):
    rng = np.random.default_rng(3)
    be = B.Backend(npd)
    x, y = rng.standard_normal(1000).astype(npd), rng.standard_normal(1000).astype(npd)
    dx, dy = _dev(x), _dev(y)
    be.blas.axpy(-2.0, dx, dy)
    np.testing.assert_allclose(dy.numpy(), y - 2 * x.astype(np.float64), rtol=tol * 4, atol=tol * 4 * 8)
    be.blas.scal(0.25, dy)
    np.testing.assert_allclose(dy.numpy(), 0.25 * (y - 2 * x.astype(np.float64)), rtol=tol * 4, atol=tol * 8)
    assert abs(be.blas.norm(dx) - np.linalg.norm(x.astype(np.float64))) <= tol * np.linalg.norm(x)
    big = np.full(64, 1e200 if npd == np.float64 else 1e30, npd)
    assert np.isfinite(be.blas.norm(_dev(big)))
    # the reference's 2-D axpy on views (vlm.cpp:141, gamma_delta[:, 1:] -= gamma[:, :-1]): (ns, nc) column-major
    ns, nc = 6, 5
    g = rng.standard_normal((nc, ns)).astype(npd)
    dg, dd = _dev(g), _dev(g.copy())
    be.blas.axpy_strided(-1.0, dg, (0, ns, nc - 1, 1, ns), dd, (ns, ns, nc - 1, 1, ns))
    want = g.astype(np.float64).copy()
    want[1:] -= g[:-1]
    np.testing.assert_allclose(dd.numpy(), want, rtol=tol, atol=tol * 4)


@pytest.mark.parametrize("npd,tol", PREC)
def test_sum_1d_and_strided_2d(cuda, npd, tol):
    rng = np.random.default_rng(4)
    be = B.Backend(npd)
    a = rng.standard_normal((9, 13)).astype(npd)
    da = _dev(a)
    assert abs(be.sum(da.view(a.size)) - a.astype(np.float64).sum()) <= tol * np.abs(a).sum()
    assert abs(be.sum(da) - a.astype(np.float64).sum()) <= tol * np.abs(a).sum()
    # a (m, n) = (13, 4) column-major view of the first 4 rows, and every other column of it
    assert abs(be.sum(da, (13, 4), (1, 13)) - a[:4].astype(np.float64).sum()) <= tol * np.abs(a).sum()
    assert abs(be.sum(da, (13, 3), (1, 26)) - a[0:6:2].astype(np.float64).sum()) <= tol * np.abs(a).sum()


@pytest.mark.parametrize("npd,tol", [(np.float32, 5e-5), (np.float64, 1e-11)])
@pytest.mark.parametrize("m,n,nrhs", [(495, 10, 1), (64, 64, 3), (200, 7, 5)])
def test_lsq_matches_numpy(cuda, npd, tol, m, n, nrhs):
    rng = np.random.default_rng(m + n)
    A = rng.standard_normal((m, n))
    Bm = rng.standard_normal((m, nrhs))
    be = B.Backend(npd)
    lsq = be.create_lsq_solver()
    dA, dB = _dev(np.ascontiguousarray(A.T).astype(npd)), _dev(np.ascontiguousarray(Bm.T).astype(npd))
    lsq.init(dA, dB)
    lsq.solve(dA, dB)
    x = dB.numpy()[:, :n].T
    want = np.linalg.lstsq(A.astype(npd).astype(np.float64), Bm.astype(npd).astype(np.float64), rcond=None)[0]
    cond = np.linalg.cond(A)
    np.testing.assert_allclose(x, want, rtol=tol * cond, atol=tol * cond * np.abs(want).max())
    # the remaining rows hold the residual's components: their norm is the residual norm
    res = np.linalg.norm(A @ want - Bm, axis=0)
    np.testing.assert_allclose(np.linalg.norm(dB.numpy()[:, n:].astype(np.float64), axis=1), res,
                               rtol=tol * cond * 10, atol=tol * cond * 10)


def test_lsq_rank_deficient_and_bad_shapes(cuda):
    be = B.Backend(np.float64)
    A = np.ones((6, 3))
    A[:, 1] = 0.0
    dA, dB = _dev(np.ascontiguousarray(A.T)), _dev(np.ones((1, 6)))
    with pytest.raises(GbvlmError, match="GBVLM_ERR_SINGULAR"):
        be.create_lsq_solver().solve(dA, dB)
    with pytest.raises(GbvlmError, match="GBVLM_ERR_ARG"):
        be.create_lsq_solver().solve(_dev(np.ones((4, 3))), _dev(np.ones((1, 3))))  # m < n
