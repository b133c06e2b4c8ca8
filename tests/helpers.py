"""Shared test helpers: input builders and tolerance checks."""
import math

import numpy as np

from tinyvlm_gb300 import mesh as M


def close(gpu, ref, rtol, atol_frac=0.0, what=""):
    """|gpu - ref| <= rtol*|ref| + atol_frac*max|ref| elementwise."""
    gpu = np.asarray(gpu, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    assert gpu.shape == ref.shape, (what, gpu.shape, ref.shape)
    scale = np.abs(ref).max() if ref.size else 0.0
    err = np.abs(gpu - ref)
    bound = rtol * np.abs(ref) + atol_frac * scale
    bad = err > bound
    if bad.any():
        i = np.unravel_index(np.argmax(err - bound), err.shape)
        raise AssertionError("%s: %d/%d entries off; worst at %s gpu=%r ref=%r (rtol=%g atol=%g)" %
                             (what, bad.sum(), bad.size, i, gpu[i], ref[i], rtol, atol_frac * scale))


def wing(kind="rect", nc=6, ns=9, dtype=np.float32):
    if kind == "rect":
        v = M.rectangular(nc, ns, chord=1.0, semispan=3.0)
    elif kind == "ellip":
        v = M.elliptic(nc, ns)
    else:
        v = M.trapezoid(nc, ns, 7.0, 0.45, 20.0)
    v = v.astype(dtype)
    M.quarter_chord(v)
    return v


def synthetic_wake(v, rows, dx=0.08, seed=0, dtype=np.float32):
    """Wake vertices (4, rows, ns+1): the TE line convected downstream with a
    small heave so the sheet is not planar; newest row last."""
    rng = np.random.default_rng(seed)
    ns1 = v.shape[2]
    te = v[:3, -1, :].astype(np.float64)
    w = np.zeros((4, rows, ns1), np.float64)
    for r in range(rows):
        age = rows - 1 - r
        w[0, r] = te[0] + dx * age
        w[1, r] = te[1] + 0.002 * age * np.sin(np.linspace(0, 1, ns1))
        w[2, r] = te[2] + 0.05 * math.sin(0.4 * age) + 0.001 * rng.standard_normal(ns1)
    w[3] = 1
    return w.astype(dtype)


def aero_inputs(v, seed=1, dtype=np.float32):
    rng = np.random.default_rng(seed)
    ns, nc = v.shape[2] - 1, v.shape[1] - 1
    g = rng.standard_normal((nc, ns)).astype(dtype)
    vel = np.empty((3, nc, ns), dtype)
    vel[0], vel[1], vel[2] = 1.0, 0.05, 0.1
    vel += 0.01 * rng.standard_normal((3, nc, ns)).astype(dtype)
    return g, vel
