"""The batched finite-difference Jacobian (CPU): same steps and columns as
scripts/finite_diff.py:26-48 on a closed-form function."""
import numpy as np

from tinyvlm_gb300.finite_diff import numerical_jac_batch, perturbed_points


def f(x):
    return np.array([np.sin(x[0]) * x[1], x[0] ** 2 + np.exp(x[2]), x[1] * x[2] ** 3])


def jac_exact(x):
    return np.array([[np.cos(x[0]) * x[1], np.sin(x[0]), 0.0],
                     [2 * x[0], 0.0, np.exp(x[2])],
                     [0.0, x[2] ** 3, 3 * x[1] * x[2] ** 2]])


def test_three_point_and_two_point():
    x = np.array([0.3, -1.7, 2.5])
    calls = []

    def fb(points):
        calls.append(len(points))
        return [f(p) for p in points]

    J3 = numerical_jac_batch(fb, x)
    J2 = numerical_jac_batch(fb, x, method="2-point")
    assert calls == [6, 4]
    np.testing.assert_allclose(J3, jac_exact(x), rtol=1e-8, atol=1e-9)
    np.testing.assert_allclose(J2, jac_exact(x), rtol=1e-6, atol=1e-6)


def test_points_follow_the_step_rule():
    x = np.array([0.0, 2.0, -3e-3])
    pts, d = perturbed_points(x)
    eps = np.finfo(np.float64).eps
    assert len(pts) == 6
    assert pts[0][0] - x[0] == eps and d[0] == 2 * eps  # h = eps at zero
    h1 = np.cbrt(eps * 2.0)  # |x| > 1
    assert np.isclose(pts[2][1] - x[1], h1, rtol=1e-12)
    h2 = np.cbrt(eps) * 3e-3
    assert np.isclose(x[2] - pts[5][2], h2, rtol=1e-9)
