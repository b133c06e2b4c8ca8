"""Finite-difference Jacobians with every column's evaluations in one batch.

Mirrors scripts/finite_diff.py:26-48 (``numerical_jac``, 3-point central
and 2-point forward): the same step sizes (``cd2_h``: max(cbrt(eps |x|) or
cbrt(eps) |x|, eps); ``fd_h``: max(sqrt(eps) |x|, eps)) and the same
representable step ``delta = xp[j] - xm[j]``.  The difference is the call
pattern: ``f_batch`` receives every perturbed point at once (2 n points for
3-point, n + 1 for 2-point), so that an HBVLM-backed residual can solve
them as one batch (``HBVLM2.run_batch`` / ``HBVLM3.run_batch``).
"""
import numpy as np

EPS = np.finfo(np.float64).eps


def fd_h(x0):
    return np.maximum(np.sqrt(EPS) * np.abs(x0), EPS)


def cd2_h(x0):
    return np.maximum(np.where(np.abs(x0) > 1, np.cbrt(EPS * np.abs(x0)), np.cbrt(EPS) * np.abs(x0)), EPS)


def perturbed_points(x, method="3-point"):
    """The points numerical_jac evaluates, in its column order, and each column's delta."""
    x = np.asarray(x, np.float64)
    n = x.size
    pts, deltas = [], np.zeros(n)
    if method == "3-point":
        for j in range(n):
            h = cd2_h(x[j])
            xp, xm = x.copy(), x.copy()
            xp[j] += h
            xm[j] -= h
            deltas[j] = xp[j] - xm[j]
            pts += [xp, xm]
    elif method == "2-point":
        pts.append(x.copy())
        for j in range(n):
            h = fd_h(x[j])
            xp = x.copy()
            xp[j] += h
            deltas[j] = xp[j] - x[j]
            pts.append(xp)
    else:
        raise ValueError("method must be '3-point' or '2-point'")
    return pts, deltas


def numerical_jac_batch(f_batch, x, *args, method="3-point"):
    """Jacobian of f at x; ``f_batch(list_of_points, *args)`` returns the list of f values."""
    pts, deltas = perturbed_points(x, method)
    vals = [np.asarray(v, np.float64) for v in f_batch(pts, *args)]
    n = len(deltas)
    jac = np.zeros((vals[0].size, n))
    if method == "3-point":
        for j in range(n):
            jac[:, j] = (vals[2 * j] - vals[2 * j + 1]) / deltas[j]
    else:
        for j in range(n):
            jac[:, j] = (vals[j + 1] - vals[0]) / deltas[j]
    return jac
