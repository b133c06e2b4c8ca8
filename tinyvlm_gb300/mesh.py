"""Planar lifting-surface meshes: plot3d I/O and parametric generators.

Vertex grids use the reference's memory layout: numpy ``(4, nc+1, ns+1)``
float arrays, i.e. the column-major ``(ns+1, nc+1, 4)`` tensor of
vlm/src/vlm.cpp:25-28 (spanwise index fastest, then chordwise, then the
x/y/z/w planes with w = 1).  Every mesh is a half wing: the solver mirrors it
in the y = 0 plane.

The plot3d reader follows vlm/src/vlm_mesh.cpp:34-123 (single block, 2-D,
chordwise rows, optional quarter-chord ring shift).  The reference ships no
mesh generator; the generators below build the planforms named by the
benchmark workloads (elliptic, rectangular, trapezoidal).
"""
import math

import numpy as np

__all__ = ["read_plot3d", "write_plot3d", "quarter_chord", "elliptic", "rectangular", "trapezoid",
           "batch_cases", "Case"]


def _finish(x, y, z, dtype):
    nc1, ns1 = x.shape
    v = np.zeros((4, nc1, ns1), dtype=dtype)
    v[0], v[1], v[2], v[3] = x, y, z, 1
    return v


def quarter_chord(v):
    """Shift every ring a quarter panel aft and extrapolate the trailing edge
    (vlm/src/vlm_mesh.cpp:16-32).  In place on a ``(4, nc+1, ns+1)`` array."""
    T = v.dtype.type
    for j in range(v.shape[1] - 1):
        v[0:3, j, :] = T(0.75) * v[0:3, j, :] + T(0.25) * v[0:3, j + 1, :]
    j = v.shape[1] - 2
    v[0:3, j + 1, :] = (T(4) / T(3)) * v[0:3, j + 1, :] - (T(1) / T(3)) * v[0:3, j, :]
    return v


def read_plot3d(path, qc=True, dtype=np.float32):
    """Read a single-block 2-D plot3d file (vlm/src/vlm_mesh.cpp:50-92)."""
    with open(path) as f:
        tok = f.read().split()
    if int(tok[0]) != 1:
        raise RuntimeError("Only single block plot3d mesh is supported")
    ni, nj, nk = int(tok[1]), int(tok[2]), int(tok[3])
    if nk != 1:
        raise RuntimeError("Only 2D plot3d mesh is supported")
    vals = np.array(tok[4:4 + 3 * ni * nj], dtype=np.float64).astype(dtype)
    v = np.zeros((4, ni, nj), dtype=dtype)
    for k in range(3):
        v[k] = vals[k * ni * nj:(k + 1) * ni * nj].reshape(nj, ni).T
    v[3] = 1
    if np.any(v[1, 1:, 0] != v[1, 0, 0]):
        raise RuntimeError("Mesh vertices should be ordered in chordwise direction")
    if qc:
        quarter_chord(v)
    return v


def write_plot3d(path, v):
    """Write ``(4 or 3, nc+1, ns+1)`` vertices as a single-block 2-D plot3d file."""
    ni, nj = v.shape[1], v.shape[2]
    with open(path, "w") as f:
        f.write("1\n%d %d 1\n" % (ni, nj))
        for k in range(3):
            vals = np.asarray(v[k], dtype=np.float64).T.ravel()
            for s in range(0, vals.size, 4):
                f.write(" ".join("%.17g" % t for t in vals[s:s + 4]) + "\n")


def elliptic(nc, ns, semispan=5.0, root_chord=1.0, dtype=np.float64):
    """Elliptic planform with a straight quarter-chord line at x = c_r/4:
    c(y) = c_r sqrt(1 - (y/s)^2), nc uniform chordwise panels and ns
    cosine-spaced spanwise panels y_k = s sin(k pi / (2 ns)).  The tip chord is
    zero, so the tip rings are triangles."""
    k = np.arange(ns + 1)
    y = semispan * np.sin(k * math.pi / (2 * ns))
    y[-1] = semispan
    c = root_chord * np.sqrt(np.clip(1.0 - (y / semispan) ** 2, 0.0, None))
    x_le = 0.25 * root_chord - 0.25 * c
    t = np.arange(nc + 1)[:, None] / nc
    x = x_le[None, :] + t * c[None, :]
    yy = np.broadcast_to(y[None, :], x.shape)
    return _finish(x, yy, np.zeros_like(x), dtype)


def rectangular(nc, ns, chord=1.0, semispan=4.0, y0=0.0, dtype=np.float64):
    """Flat rectangular half wing (the reference's ``infinite_rectangular``
    meshes are this with a semispan of 40000)."""
    x = np.broadcast_to((np.arange(nc + 1) / nc * chord)[:, None], (nc + 1, ns + 1))
    y = np.broadcast_to((y0 + np.arange(ns + 1) / ns * semispan)[None, :], (nc + 1, ns + 1))
    return _finish(np.array(x), np.array(y), np.zeros((nc + 1, ns + 1)), dtype)


def trapezoid(nc, ns, aspect_ratio, taper, sweep_deg, root_chord=1.0, dtype=np.float64):
    """Trapezoidal half wing: semispan s = AR (1 + taper) c_r / 4 so that the
    full wing has aspect ratio AR; leading edge swept by ``sweep_deg``; chord
    c(y) = c_r (1 - (1 - taper) y / s); uniform panels both ways."""
    s = aspect_ratio * (1.0 + taper) * root_chord / 4.0
    y = np.arange(ns + 1) / ns * s
    c = root_chord * (1.0 - (1.0 - taper) * y / s)
    x_le = y * math.tan(math.radians(sweep_deg))
    t = np.arange(nc + 1)[:, None] / nc
    x = x_le[None, :] + t * c[None, :]
    yy = np.broadcast_to(y[None, :], x.shape)
    return _finish(x, np.array(yy), np.zeros_like(x), dtype)


class Case:
    """One batched steady case: a half wing and its angles of attack."""

    def __init__(self, verts, alphas, params):
        self.verts = verts
        self.alphas = alphas
        self.params = params

    @property
    def ns(self):
        return self.verts.shape[2] - 1

    @property
    def nc(self):
        return self.verts.shape[1] - 1

    @property
    def n(self):
        return self.ns * self.nc


def batch_cases(count=512, seed=20261203, n_alpha=8, nc_range=(4, 32), ns_range=(4, 64),
                ar_range=(4.0, 12.0), taper_range=(0.3, 1.0), sweep_range=(0.0, 35.0),
                alpha_deg_range=(-8.0, 8.0), qc=True, dtype=np.float32):
    """Seeded uneven batch of trapezoidal half wings (numpy PCG64).

    Each case draws nc ~ U{4..32}, ns ~ U{4..64}, AR ~ U[4, 12],
    taper ~ U[0.3, 1], LE sweep ~ U[0, 35] degrees and ``n_alpha`` angles of
    attack ~ U[-8, 8] degrees (returned in radians).  Vertices get the
    quarter-chord shift the plot3d reader applies."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cases = []
    for _ in range(count):
        nc = int(rng.integers(nc_range[0], nc_range[1] + 1))
        ns = int(rng.integers(ns_range[0], ns_range[1] + 1))
        ar = float(rng.uniform(*ar_range))
        lam = float(rng.uniform(*taper_range))
        sw = float(rng.uniform(*sweep_range))
        al = np.radians(rng.uniform(alpha_deg_range[0], alpha_deg_range[1], size=n_alpha))
        v = trapezoid(nc, ns, ar, lam, sw, dtype=np.float64).astype(dtype)
        if qc:
            quarter_chord(v)
        cases.append(Case(v, al.astype(np.float64), dict(nc=nc, ns=ns, ar=ar, taper=lam, sweep=sw)))
    return cases
