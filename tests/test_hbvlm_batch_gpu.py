"""HBVLM over K parameter sets at once (the finite-difference Jacobian
columns of the continuation scripts): each set equals its own single run and
the oracle; the batched Jacobian equals the column-by-column one."""
import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.finite_diff import numerical_jac_batch, perturbed_points
from tinyvlm_gb300.hbvlm import HBVLM2, HBVLM3

pytestmark = pytest.mark.gpu


def section(nc, x0, x1, semispan=10000.0):
    v = M.rectangular(nc, 1, x1 - x0, semispan)
    v[0] += x0
    return v


def _sets2(K, H, seed):
    rng = np.random.default_rng(seed)
    oms = list(rng.uniform(0.35, 0.5, K))
    dyns = []
    for _ in range(K):
        d = np.zeros((2, 2 * H + 1))
        d[0, 1:3] = rng.uniform(-0.02, 0.02, 2)
        d[1, 0] = rng.uniform(-0.02, 0.02)
        d[1, 1:3] = rng.uniform(-0.04, 0.04, 2)
        dyns.append(d)
    return oms, dyns


def test_hbvlm2_batch_equals_single_runs(cuda):
    v = M.rectangular(10, 1, 1.0, 40000.0)
    H, K = 2, 5
    oms, dyns = _sets2(K, H, 11)
    hb = HBVLM2("gb300", v)
    hb.init(H, 1.0)
    fl = [np.zeros((2, 2 * H + 1)) for _ in range(K)]
    hb.run_batch(oms, dyns, fl)
    its = list(hb.iterations)
    last = hb.gamma_coeffs.copy()
    for k in range(K):
        hb.gamma_coeffs[:] = 0.0
        ft = np.zeros((2, 2 * H + 1))
        hb.run(oms[k], dyns[k], ft)
        print(k, "batch iterations", its[k], "single", hb.iterations, "max diff", np.abs(ft - fl[k]).max())
        np.testing.assert_allclose(fl[k], ft, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(last, hb.gamma_coeffs, rtol=1e-9, atol=1e-12)


def test_hbvlm3_batch_matches_oracle(cuda):
    wing = section(9, 0.0, 0.1905)
    flap = section(3, 0.1905, 0.254)
    hb = HBVLM3("gb300", [wing, flap])
    hb.init(2, 1.0 / 0.127)
    x0 = hb.gamma_coeffs.copy()
    base = np.array([[0.0, 0.01, 0.0, 0.0, 0.0], [0.02, 0.0, 0.03, 0.0, 0.0], [0.0, 0.01, 0.0, 0.005, 0.0]])
    dyns = [base, base * 1.1, base + 0.002]
    oms, Us = [1.0, 0.9, 1.1], [10.0, 10.0, 9.5]
    fl = [np.zeros((3, 5)) for _ in range(3)]
    hb.run_batch(oms, Us, dyns, fl)
    for k, L in enumerate(hb._last_batch):
        X, out, it = O.hbvlm_run(hb.verts, [False, True], 2, oms[k], L["dt"], L["max_t"], L["wake_T"], L["inst"],
                                 L["dft"], L["ddft"], L["finst"], L["fs"], L["ref_a"], L["ref_b"], True, x0, 1e-12)
        print(k, "gpu iterations", hb.iterations[k], "oracle", it, "max diff", np.abs(fl[k] - out).max())
        np.testing.assert_allclose(fl[k], out, rtol=1e-8, atol=1e-10)


def test_fd_jacobian_batch_equals_columnwise(cuda):
    """The 3-point Jacobian of the 2-DOF HBVLM loads with respect to the motion
    coefficients: every perturbed point in one batch against one run per point
    (each from the same starting coefficients)."""
    v = M.rectangular(8, 1, 1.0, 40000.0)
    H = 1
    hb = HBVLM2("gb300", v)
    hb.init(H, 1.0)
    omega = 0.45
    x = np.array([0.005, 0.02, -0.01, 0.01, 0.03, 0.015])  # motion coefficients (2 x 3), flattened

    def f_batch(points):
        fl = [np.zeros((2, 2 * H + 1)) for _ in points]
        hb.gamma_coeffs[:] = 0.0
        hb.run_batch([omega] * len(points), [p.reshape(2, -1) for p in points], fl)
        return [f.ravel() for f in fl]

    J = numerical_jac_batch(f_batch, x)
    pts, deltas = perturbed_points(x)
    cols = []
    for p in pts:
        hb.gamma_coeffs[:] = 0.0
        ft = np.zeros((2, 2 * H + 1))
        hb.run(omega, p.reshape(2, -1), ft)
        cols.append(ft.ravel())
    J1 = np.stack([(cols[2 * j] - cols[2 * j + 1]) / deltas[j] for j in range(len(deltas))], axis=1)
    print("jacobian max", np.abs(J1).max(), "diff", np.abs(J - J1).max())
    assert np.abs(J1).max() > 1e-3
    # a set's operator, iteration and solve do not depend on the rest of the batch
    np.testing.assert_allclose(J, J1, rtol=1e-9, atol=1e-9 * np.abs(J1).max())


def test_device_wake_transforms_match_host(cuda):
    """The wake transforms evaluated on the device from the chain parameters
    against the host closed form (bitwise the dual-number tree): the same map
    to rounding, for the 3-DOF chain (flap after the pitch)."""
    wing = section(9, 0.0, 0.1905)
    flap = section(3, 0.1905, 0.254)
    hb = HBVLM3("gb300", [wing, flap])
    hb.init(2, 1.0 / 0.127)
    dyn = np.array([[0.0, 0.01, 0.0, 0.0, 0.0], [0.02, 0.0, 0.03, 0.0, 0.0], [0.0, 0.01, 0.0, 0.005, 0.0]])
    hb.run(1.0, 10.0, dyn, np.zeros((3, 5)))
    L = hb._last
    x = np.asfortranarray(np.random.default_rng(5).standard_normal((hb.engine.n, 5)) * 0.01)
    y_dev = hb.engine.map(x, 1.0, L["dt"])
    ts, tm, T, Td = L["inst"]
    hb.engine.prepare_batch(2, [L["max_t"]], [L["wake_T"]], ts, tm, T, Td, [L["dft"]])
    y_host = hb.engine.map(x, 1.0, L["dt"])
    print("device vs host wake transforms: map diff", np.abs(y_dev - y_host).max(), np.abs(y_host).max())
    np.testing.assert_allclose(y_dev, y_host, rtol=1e-12, atol=1e-15)
