"""Oracle (test infrastructure only): CPU restatement of the tinyvlm
vortex-lattice hot path, used by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker.  The product never
imports this module.

Heavy per-element kernels run in C (``vlm_oracle.c``, built by ``build.py``);
the drivers below restate the reference's simulation drivers in numpy, and the
dense factor/solve calls LAPACK ``?getrf/?getrs`` through scipy -- the same
LAPACK routines the reference's CPU backend calls through LAPACKE
(vlm/backends/cpu/src/vlm_backend_cpu_lapack.cpp:40-94; scipy bundles
OpenBLAS, the reference pins OpenBLAS 0.3.26/0.3.29 in packages/openblas.lua).

Array conventions (identical memory layout to the reference's column-major
tensors, vlm/include/vlm_memory.hpp:306-319):
  wing vertices  numpy (4, nc+1, ns+1)  == reference (ns+1, nc+1, 4)
  panel vectors  numpy (3, nc, ns)      == reference (ns, nc, 3)
  panel scalars  numpy (nc, ns)         == reference (ns, nc)
  wake vertices  numpy (4, nwv, ns+1)   == reference (ns+1, nwv, 4)
  wake gamma     numpy (nwv-1, ns)      == reference (ns, nwv-1)
  LHS            numpy (n, n) Fortran order, A[row=colloc, col=ring]
"""
import ctypes
import math
import os

import numpy as np

from . import build as _build

_lib = None

PI_F = np.float32(3.141593)  # vlm/include/vlm_types.hpp:22


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        for pre, ct in (("f", ctypes.c_float), ("d", ctypes.c_double)):
            P = ctypes.c_void_p
            I64, I32 = ctypes.c_int64, ctypes.c_int32
            getattr(L, "orc_sum_" + pre).restype = ct
            getattr(L, "orc_mesh_mac_" + pre).restype = ct
            getattr(L, "orc_coeff_cl_" + pre).restype = ct
            getattr(L, "orc_trefftz_cd_" + pre).restype = ct
            getattr(L, "orc_trefftz_cd_" + pre).argtypes = [P, I64, I64, I64, P, ct]
            getattr(L, "orc_influence_" + pre).argtypes = [I64, P, P, I64, P, I64, I64, P, I64, ct]
            getattr(L, "orc_wake_influence_" + pre).argtypes = [P, I64, P, I64, P, I64, I64, I64, P, P, ct, I32]
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _sfx(dtype):
    return "f" if np.dtype(dtype) == np.float32 else "d"


def _ct(dtype):
    return ctypes.c_float if np.dtype(dtype) == np.float32 else ctypes.c_double


def _p(a):
    assert a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def _parr(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def _i64(vals):
    return (ctypes.c_int64 * len(vals))(*vals)


def _i32(vals):
    return (ctypes.c_int32 * len(vals))(*vals)


def num_threads():
    return lib().orc_num_threads()


# ---------------------------------------------------------------------------
# flow data, vlm/src/vlm_utils.cpp:5-19, vlm/src/vlm_data.cpp:8-13
# ---------------------------------------------------------------------------
def freestream(u_inf, alpha, beta, dtype=np.float32):
    T = np.dtype(dtype).type
    u, a, b = T(u_inf), T(alpha), T(beta)
    return np.array([u * np.cos(a) * np.cos(b), -(u * np.cos(a) * np.sin(b)), u * np.sin(a)], dtype=dtype)


def lift_axis(fs):
    T = fs.dtype.type
    c = np.array([fs[1] * T(0) - fs[2] * T(1), fs[2] * T(0) - fs[0] * T(0), fs[0] * T(1) - fs[1] * T(0)], dtype=fs.dtype)
    return c / np.sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])


def translation(t, dtype):
    """Column-major 4x4 translation (vlm/include/vlm_kinematics.hpp translation_matrix)."""
    m = np.eye(4, dtype=dtype)
    m[0:3, 3] = t
    return np.asfortranarray(m)


# ---------------------------------------------------------------------------
# plot3d reader and quarter-chord shift, vlm/src/vlm_mesh.cpp:16-92
# ---------------------------------------------------------------------------
def read_plot3d(path, qc=True, dtype=np.float32):
    tok = open(path).read().split()
    if int(tok[0]) != 1:
        raise RuntimeError("Only single block plot3d mesh is supported")
    ni, nj, nk = int(tok[1]), int(tok[2]), int(tok[3])
    if nk != 1:
        raise RuntimeError("Only 2D plot3d mesh is supported")
    vals = np.array(tok[4:4 + 3 * ni * nj], dtype=np.float64).astype(dtype)
    v = np.zeros((4, ni, nj), dtype=dtype)  # reference (nj, ni, 4): span index fastest
    for k in range(3):
        v[k] = vals[k * ni * nj:(k + 1) * ni * nj].reshape(nj, ni).T
    v[3] = 1
    if np.any(v[1, 1:, 0] != v[1, 0, 0]):
        raise RuntimeError("Mesh vertices should be ordered in chordwise direction")
    if qc:
        quarter_chord(v)
    return v


def quarter_chord(v):
    """vlm_mesh.cpp:16-32, in place on (4, nc+1, ns+1)."""
    T = v.dtype.type
    for j in range(v.shape[1] - 1):
        v[0:3, j, :] = T(0.75) * v[0:3, j, :] + T(0.25) * v[0:3, j + 1, :]
    j = v.shape[1] - 2
    v[0:3, j + 1, :] = (T(4) / T(3)) * v[0:3, j + 1, :] - (T(1) / T(3)) * v[0:3, j, :]


# ---------------------------------------------------------------------------
# Backend operators (thin wrappers over the C restatement)
# ---------------------------------------------------------------------------
def dims(verts):
    return [v.shape[2] - 1 for v in verts], [v.shape[1] - 1 for v in verts]


def mesh_metrics(alpha, verts, dtype):
    T = np.dtype(dtype).type
    out = []
    for v in verts:
        ns, nc = v.shape[2] - 1, v.shape[1] - 1
        col = np.zeros((3, nc, ns), dtype)
        nor = np.zeros((3, nc, ns), dtype)
        ar = np.zeros((nc, ns), dtype)
        getattr(lib(), "orc_mesh_metrics_" + _sfx(dtype))(_ct(dtype)(T(alpha)), ctypes.c_int64(ns), ctypes.c_int64(nc),
                                                          _p(v), _p(col), _p(nor), _p(ar))
        out.append((col, nor, ar))
    return [o[0] for o in out], [o[1] for o in out], [o[2] for o in out]


def lhs_assemble(lhs, colloc, normals, verts_wing, verts_wake, iteration, sigma=0.0):
    dt = lhs.dtype
    ns, nc = dims(verts_wing)
    nwv = [w.shape[1] for w in verts_wake]
    getattr(lib(), "orc_lhs_assemble_" + _sfx(dt))(
        _p(lhs), ctypes.c_int64(lhs.shape[0]), ctypes.c_int32(len(ns)), _i64(ns), _i64(nc), _i64(nwv),
        _parr(colloc), _parr(normals), _parr(verts_wing), _parr(verts_wake), ctypes.c_int32(iteration),
        _ct(dt)(sigma))


def rhs_assemble_velocities(rhs, normals, velocities):
    ns = [n.shape[2] for n in normals]
    nc = [n.shape[1] for n in normals]
    getattr(lib(), "orc_rhs_assemble_velocities_" + _sfx(rhs.dtype))(
        _p(rhs), ctypes.c_int32(len(ns)), _i64(ns), _i64(nc), _parr(normals), _parr(velocities))


def rhs_assemble_wake_influence(rhs, gamma_wake, colloc, normals, verts_wake, lifting, iteration, sigma=0.0):
    ns = [n.shape[2] for n in normals]
    nc = [n.shape[1] for n in normals]
    nwv = [w.shape[1] for w in verts_wake]
    getattr(lib(), "orc_rhs_assemble_wake_influence_" + _sfx(rhs.dtype))(
        _p(rhs), ctypes.c_int32(len(ns)), _i64(ns), _i64(nc), _i64(nwv), _parr(gamma_wake), _parr(colloc),
        _parr(normals), _parr(verts_wake), _i32([1 if l else 0 for l in lifting]), ctypes.c_int32(iteration),
        _ct(rhs.dtype)(sigma))


def wake_rollup(verts_wake, verts_wing, gamma_wing, gamma_wake, lifting, dt, iteration, sigma=0.0):
    d = verts_wake[0].dtype
    ns, nc = dims(verts_wing)
    nwv = [w.shape[1] for w in verts_wake]
    scratch = [w.copy() for w in verts_wake]
    getattr(lib(), "orc_wake_rollup_" + _sfx(d))(
        ctypes.c_int32(len(ns)), _i64(ns), _i64(nc), _i64(nwv), _parr(verts_wake), _parr(verts_wing),
        _parr(gamma_wing), _parr(gamma_wake), _parr(scratch), _i32([1 if l else 0 for l in lifting]),
        _ct(d)(sigma), _ct(d)(dt), ctypes.c_int32(iteration))


def forces_steady(verts, gamma_delta, velocities):
    d = verts.dtype
    nc, ns = gamma_delta.shape
    f = np.zeros((3, nc, ns), d)
    getattr(lib(), "orc_forces_steady_" + _sfx(d))(ctypes.c_int64(ns), ctypes.c_int64(nc), _p(verts),
                                                   _p(gamma_delta), _p(velocities), _p(f))
    return f


def forces_unsteady(verts, gamma_delta, dgamma_dt, velocities, areas, normals):
    d = verts.dtype
    nc, ns = gamma_delta.shape
    f = np.zeros((3, nc, ns), d)
    getattr(lib(), "orc_forces_unsteady_" + _sfx(d))(ctypes.c_int64(ns), ctypes.c_int64(nc), _p(verts),
                                                     _p(gamma_delta), _p(dgamma_dt), _p(velocities), _p(areas),
                                                     _p(normals), _p(f))
    return f


def coeff_cl(forces, lift, fs, rho, area):
    d = forces.dtype
    _, nc, ns = forces.shape
    T = d.type
    return T(getattr(lib(), "orc_coeff_cl_" + _sfx(d))(ctypes.c_int64(ns), ctypes.c_int64(nc), _p(forces),
                                                       _p(np.ascontiguousarray(lift, d)),
                                                       _p(np.ascontiguousarray(fs, d)), _ct(d)(rho), _ct(d)(area)))


def coeff_cm(forces, verts, ref_pt, fs, rho, area, mac):
    d = forces.dtype
    _, nc, ns = forces.shape
    out = np.zeros(3, d)
    getattr(lib(), "orc_coeff_cm_" + _sfx(d))(ctypes.c_int64(ns), ctypes.c_int64(nc), _p(forces), _p(verts),
                                              _p(np.ascontiguousarray(ref_pt, d)), _p(np.ascontiguousarray(fs, d)),
                                              _ct(d)(rho), _ct(d)(area), _ct(d)(mac), _p(out))
    return out


def asum(x):
    d = x.dtype
    return d.type(getattr(lib(), "orc_sum_" + _sfx(d))(ctypes.c_int64(x.size), _p(x)))


def mesh_mac(verts, areas):
    d = verts.dtype
    nc, ns = areas.shape
    return d.type(getattr(lib(), "orc_mesh_mac_" + _sfx(d))(ctypes.c_int64(ns), ctypes.c_int64(nc), _p(verts), _p(areas)))


def trefftz_cd(verts_wake, gamma_wake, sigma=0.0):
    d = verts_wake.dtype
    _, nwv, n = verts_wake.shape
    return d.type(getattr(lib(), "orc_trefftz_cd_" + _sfx(d))(_p(verts_wake), n * nwv, nwv, n, _p(gamma_wake),
                                                              _ct(d)(sigma)))


def gamma_wake_from_coeffs(gamma_wake, coeffs, harmonics, tn, omega, dt, iteration):
    d = gamma_wake.dtype
    ncols, ns = gamma_wake.shape
    T = d.type
    getattr(lib(), "orc_gamma_wake_from_coeffs_" + _sfx(d))(
        ctypes.c_int64(ns), ctypes.c_int64(ncols), _p(gamma_wake), _p(np.asfortranarray(coeffs, d)),
        ctypes.c_int32(harmonics), _ct(d)(T(tn)), _ct(d)(T(omega)), _ct(d)(T(dt)), ctypes.c_int64(iteration))


def displace_wing(transform, verts, verts_init):
    d = verts.dtype
    nv = verts.shape[1] * verts.shape[2]
    getattr(lib(), "orc_displace_wing_" + _sfx(d))(ctypes.c_int64(nv), _p(np.asfortranarray(transform, d)),
                                                   _p(verts), _p(verts_init))


def wake_shed(verts_wing, verts_wake, iteration):
    """vlm/src/vlm_backend.cpp:43-47: wing TE vertex row -> wake row -1-iteration."""
    for w, k in zip(verts_wing, verts_wake):
        k[:, k.shape[1] - 1 - iteration, :] = w[:, -1, :]


def lu_factor(A):
    """LAPACK ?getrf (vlm_backend_cpu_lapack.cpp:40-50)."""
    from scipy.linalg import lapack
    f = lapack.sgetrf if A.dtype == np.float32 else lapack.dgetrf
    lu, piv, info = f(A, overwrite_a=True)
    if info != 0:
        raise RuntimeError("getrf failed: info=%d" % info)
    return lu, piv


def lu_solve(lu, piv, b):
    """LAPACK ?getrs (vlm_backend_cpu_lapack.cpp:52-64)."""
    from scipy.linalg import lapack
    f = lapack.sgetrs if lu.dtype == np.float32 else lapack.dgetrs
    x, info = f(lu, piv, b)
    if info != 0:
        raise RuntimeError("getrs failed: info=%d" % info)
    return x


# ---------------------------------------------------------------------------
# Multibody coefficient reductions, vlm/src/vlm_backend.cpp:72-139
# ---------------------------------------------------------------------------
def coeff_cl_multibody(forces, areas, fs, rho):
    T = fs.dtype.type
    cl, total = T(0), T(0)
    la = lift_axis(fs)
    for f, a in zip(forces, areas):
        area = asum(a)
        cl += coeff_cl(f, la, fs, rho, area) * area
        total += area
    return T(cl / total)


def coeff_cm_multibody(forces, verts, areas, ref_pt, fs, rho):
    T = fs.dtype.type
    cm = np.zeros(3, fs.dtype)
    ta, tm = T(0), T(0)
    for f, v, a in zip(forces, verts, areas):
        area = asum(a)
        mac = mesh_mac(v, a)
        cm += coeff_cm(f, v, ref_pt, fs, rho, area, mac) * area * mac
        ta += area
        tm += mac
    return cm / (ta * tm)


def gamma_delta(gamma):
    """Chordwise delta (vlm/src/vlm.cpp:138-140): d[:, 1:] = g[:, 1:] - g[:, :-1]."""
    d = gamma.copy()
    d[1:, :] -= gamma[:-1, :]
    return d


# ---------------------------------------------------------------------------
# Steady VLM driver, vlm/src/vlm.cpp:60-151 (plus CDi and CM outputs)
# ---------------------------------------------------------------------------
def vlm_run(verts_init, alpha, beta=0.0, u_inf=1.0, rho=1.0, dtype=np.float32, sigma=0.0,
            ref_pt=(0.0, 0.0, 0.0), return_state=False):
    """One steady solve with the reference's semantics.

    Returns dict(cl, cdi, cm, gamma) where gamma is a list of (nc, ns) arrays.
    CL follows VLM::run.  CDi is the Trefftz-plane drag of the (dead in the
    reference) kernel_trefftz_cd normalised as its commented caller does,
    area-weighted over surfaces like CL; CM is coeff_cm_multibody about
    ``ref_pt`` in the wing's own frame (VLM::run leaves CM at zero).
    """
    T = np.dtype(dtype).type
    verts_init = [np.ascontiguousarray(v, dtype) for v in verts_init]
    verts = [v.copy() for v in verts_init]
    ns, nc = dims(verts)
    n = sum(a * b for a, b in zip(ns, nc))
    fs = freestream(u_inf, alpha, beta, dtype)
    wake = []
    for s in ns:
        w = np.zeros((4, 2, s + 1), dtype)
        w[3] = 1
        wake.append(w)
    a32 = T(alpha)
    tr = translation(np.array([T(-100.0) * T(u_inf) * np.cos(a32), T(0), T(-100.0) * T(u_inf) * np.sin(a32)], dtype),
                     dtype)
    wake_shed(verts, wake, 0)
    for v, vi in zip(verts, verts_init):
        displace_wing(tr, v, vi)
    wake_shed(verts, wake, 1)
    colloc, normals, areas = mesh_metrics(alpha, verts, dtype)
    lhs = np.zeros((n, n), dtype, order="F")
    lhs_assemble(lhs, colloc, normals, verts, wake, 1, sigma)
    vel = []
    for s, c in zip(ns, nc):
        v = np.empty((3, c, s), dtype)
        v[0], v[1], v[2] = fs[0], fs[1], fs[2]
        vel.append(v)
    rhs = np.zeros(n, dtype)
    rhs_assemble_velocities(rhs, normals, vel)
    A = lhs.copy(order="F") if return_state else lhs
    lu, piv = lu_factor(A)
    x = lu_solve(lu, piv, rhs)
    gam, deltas, gwake = [], [], []
    off = 0
    for s, c in zip(ns, nc):
        g = x[off:off + s * c].reshape(c, s).copy()
        off += s * c
        gam.append(g)
        deltas.append(gamma_delta(g))
        gw = np.zeros((1, s), dtype)
        gw[0] = g[-1]
        gwake.append(gw)
    forces = [forces_steady(v, d, u) for v, d, u in zip(verts, deltas, vel)]
    cl = coeff_cl_multibody(forces, areas, fs, T(rho))
    # the wing sits displaced by the wake translation; the moment reference
    # moves with it, so CM is the body-frame moment about ref_pt
    ref_disp = np.asarray(ref_pt, dtype) + tr[0:3, 3]
    cm = coeff_cm_multibody(forces, verts, areas, ref_disp, fs, T(rho))
    cdi_num, area_tot = T(0), T(0)
    for w, gw, a in zip(wake, gwake, areas):
        area = asum(a)
        cdi_num += trefftz_cd(w, gw, sigma) / (np.dot(fs, fs) * area) * area
        area_tot += area
    out = dict(cl=cl, cdi=T(cdi_num / area_tot), cm=cm, gamma=gam)
    if return_state:
        out.update(lhs=lhs, rhs=rhs, colloc=colloc, normals=normals, areas=areas, verts=verts, wake=wake,
                   forces=forces)
    return out


# ---------------------------------------------------------------------------
# Shared-AIC steady sweep: one AIC per wing at alpha = 0 (collocation factor
# 1/2, 100-chord wake along +x), every alpha a right-hand side.  Built from
# the same operators as vlm_run; the reference's LU::solve takes several
# right-hand sides (vlm_backend_cpu_lapack.cpp:52-64).
# ---------------------------------------------------------------------------
def vlm_shared(verts_init, alphas, u_inf=1.0, rho=1.0, dtype=np.float64, ref_pt=(0.0, 0.0, 0.0), sigma=0.0):
    T = np.dtype(dtype).type
    r0 = vlm_run(verts_init, 0.0, 0.0, u_inf, rho, dtype, sigma, ref_pt, return_state=True)
    lhs, normals, areas, verts, wake = r0["lhs"], r0["normals"], r0["areas"], r0["verts"], r0["wake"]
    ns, nc = dims(verts)
    lu, piv = lu_factor(lhs.copy(order="F"))
    tr = translation(np.array([T(-100.0) * T(u_inf), T(0), T(0)], dtype), dtype)
    ref_disp = np.asarray(ref_pt, dtype) + tr[0:3, 3]
    out = []
    for al in alphas:
        fs = freestream(u_inf, al, 0.0, dtype)
        vel = []
        for s, c in zip(ns, nc):
            v = np.empty((3, c, s), dtype)
            v[0], v[1], v[2] = fs[0], fs[1], fs[2]
            vel.append(v)
        rhs = np.zeros(sum(a * b for a, b in zip(ns, nc)), dtype)
        rhs_assemble_velocities(rhs, normals, vel)
        x = lu_solve(lu, piv, rhs)
        gam, deltas, gwake, off = [], [], [], 0
        for s, c in zip(ns, nc):
            g = x[off:off + s * c].reshape(c, s).copy()
            off += s * c
            gam.append(g)
            deltas.append(gamma_delta(g))
            gw = np.zeros((1, s), dtype)
            gw[0] = g[-1]
            gwake.append(gw)
        forces = [forces_steady(v, d, u) for v, d, u in zip(verts, deltas, vel)]
        cl = coeff_cl_multibody(forces, areas, fs, T(rho))
        cm = coeff_cm_multibody(forces, verts, areas, ref_disp, fs, T(rho))
        cdn, at = T(0), T(0)
        for w, gw, a in zip(wake, gwake, areas):
            area = asum(a)
            cdn += trefftz_cd(w, gw, sigma) / (np.dot(fs, fs) * area) * area
            at += area
        out.append(dict(cl=cl, cdi=T(cdn / at), cm=cm, gamma=gam))
    return out


# ---------------------------------------------------------------------------
# UVLM driver, vlm/src/vlm.cpp:358-509, over precomputed per-step transforms
# T[i, m] (16, column-major), Td[i, m], freestream fs[i], reference ref[i]
# (the same arrays the GPU driver receives).
# ---------------------------------------------------------------------------
def uvlm_run(verts_init, lifting, T, Td, fs, ref, t_steps, dt, dtype=np.float64, rollup=False, sigma=0.0):
    dt_ = np.dtype(dtype).type
    verts_init = [np.ascontiguousarray(v, dtype) for v in verts_init]
    ns, nc = dims(verts_init)
    nsurf = len(verts_init)
    n = sum(a * b for a, b in zip(ns, nc))
    tr = lambda i, m: np.asfortranarray(np.asarray(T[i, m], dtype).reshape(4, 4).T)
    vpos = [v.copy() for v in verts_init]
    for m in range(nsurf):
        displace_wing(tr(0, m), vpos[m], verts_init[m])
    verts = [v.copy() for v in vpos]
    colloc, normals, areas = mesh_metrics(0.0, verts, dtype)
    colloc0 = [c.copy() for c in colloc]
    wake = []
    for s in ns:
        w = np.zeros((4, t_steps, s + 1), dtype)
        w[3] = 1
        wake.append(w)
    gwake = [np.zeros((t_steps - 1, s), dtype) for s in ns]
    lhs = np.zeros((n, n), dtype, order="F")
    lhs_assemble(lhs, colloc, normals, verts, wake, 0, sigma)
    lu, piv = lu_factor(lhs)
    gprev = [np.zeros((c, s), dtype) for s, c in zip(ns, nc)]
    cl = np.zeros(t_steps)
    cm = np.zeros((t_steps, 3))
    gam = None
    for i in range(t_steps - 1):
        wake_shed(verts, wake, i)
        vel = []
        for m in range(nsurf):
            d = np.asarray(Td[i, m], np.float64).reshape(4, 4).T.astype(dtype)
            c = colloc0[m]
            v = np.empty_like(c)
            for r in range(3):
                v[r] = -(d[r, 0] * c[0] + d[r, 1] * c[1] + d[r, 2] * c[2] + d[r, 3])
            vel.append(v)
        rhs = np.zeros(n, dtype)
        rhs_assemble_velocities(rhs, normals, vel)
        rhs_assemble_wake_influence(rhs, gwake, colloc, normals, wake, lifting, i, sigma)
        x = lu_solve(lu, piv, rhs)
        gam, deltas, gdts, off = [], [], [], 0
        for m in range(nsurf):
            g = x[off:off + ns[m] * nc[m]].reshape(nc[m], ns[m]).copy()
            off += ns[m] * nc[m]
            gam.append(g)
            deltas.append(gamma_delta(g))
            gwake[m][t_steps - 2 - i] = g[-1]
            gdts.append(((g - gprev[m]) * dt_(1.0 / dt)).astype(dtype) if dtype == np.float64 else
                        ((g - gprev[m]) * (dt_(1) / dt_(dt))).astype(dtype))
        if i > 0:
            forces = [forces_unsteady(verts[m], deltas[m], gdts[m], vel[m], areas[m], normals[m])
                      for m in range(nsurf)]
            f_s = np.asarray(fs[i], dtype)
            cl[i] = coeff_cl_multibody(forces, areas, f_s, dt_(1))
            cm[i] = coeff_cm_multibody(forces, verts, areas, np.asarray(ref[i], dtype), f_s, dt_(1))
        if rollup and i > 0:
            wake_rollup(wake, verts, gam, gwake, lifting, dt, i, sigma)
        gprev = [g.copy() for g in gam]
        for m in range(nsurf):
            displace_wing(tr(i + 1, m), verts[m], vpos[m])
        colloc, normals, areas = mesh_metrics(0.0, verts, dtype)
    return dict(cl=cl, cm=cm, gamma=gam)


# ---------------------------------------------------------------------------
# Anderson acceleration, vlm/src/vlm_solvers.cpp:6-115 (type II, history m;
# least squares through LAPACK ?gels like the CPU LSQ, vlm_backend_cpu_lapack.cpp:123-205)
# ---------------------------------------------------------------------------
def anderson(x0, f, max_iter=100, tol=1e-6, m=3):
    from scipy.linalg import lapack
    x_curr = np.array(x0, np.float64)
    n = x_curr.size
    X = np.zeros((n, m))
    G = np.zeros((n, m))
    x_new = f(x_curr)
    g_curr = x_new - x_curr
    X[:, 0] = g_curr
    x_curr = x_new
    x_new = f(x_curr)
    g_new = x_new - x_curr
    G[:, 0] = g_new - g_curr
    g_curr = g_new
    k = 1
    while k < max_iter and np.linalg.norm(g_curr) > tol:
        mk = min(m, k)
        A = np.asfortranarray(G[:, :mk].copy())
        b = g_curr.copy().reshape(-1, 1)
        _, sol, info = lapack.dgels(A, b)
        gam = sol[:mk, 0]
        x_new = x_curr + g_curr - X[:, :mk] @ gam - G[:, :mk] @ gam
        X[:, k % m] = x_new - x_curr
        x_curr = x_new
        x_new = f(x_curr)
        g_new = x_new - x_curr
        G[:, k % m] = g_new - g_curr
        g_curr = g_new
        k += 1
    return x_curr, k


# ---------------------------------------------------------------------------
# Harmonic-balance VLM, lib/libhbvlm3.cpp:262-552 (double), over the host
# arrays the product's HBVLM module builds (kinematics, DFT, instances).
# ---------------------------------------------------------------------------
def hbvlm_run(verts, lifting, H, omega, dt, max_t, wake_T, inst, dft, ddft, force_inst, fs, ref_a, ref_b,
              coupled_te, x0, tol, m=10, max_iter=100):
    dtp = np.float64
    verts_init = [np.ascontiguousarray(v, dtp) for v in verts]
    ns, nc = dims(verts_init)
    nsurf = len(verts_init)
    N = 2 * H + 1
    n = sum(a * b for a, b in zip(ns, nc))
    poff = np.cumsum([0] + [a * b for a, b in zip(ns, nc)])
    w = lifting.index(True)
    tr = lambda A, i, mm: np.asfortranarray(np.asarray(A[i, mm]).reshape(4, 4).T)
    vcur = [v.copy() for v in verts_init]
    colloc_h, normals0, _ = mesh_metrics(0.0, vcur, dtp)
    wake = []
    for s in ns:
        wk = np.zeros((4, max_t, s + 1), dtp)
        wk[3] = 1
        wake.append(wk)
    lhs = np.zeros((n, n), dtp, order="F")
    lhs_assemble(lhs, colloc_h, normals0, vcur, wake, 0)
    lu, piv = lu_factor(lhs)
    for i in range(max_t):
        for mm in range(nsurf):
            displace_wing(tr(wake_T, i, mm), vcur[mm], verts_init[mm])
        wake_shed(vcur, wake, i)

    def vel_of(Td, i, c0):
        out = []
        for mm in range(nsurf):
            d = np.asarray(Td[i, mm]).reshape(4, 4).T
            c = c0[mm]
            v = np.empty_like(c)
            for r in range(3):
                v[r] = -(d[r, 0] * c[0] + d[r, 1] * c[1] + d[r, 2] * c[2] + d[r, 3])
            out.append(v)
        return out

    ts, tm, T, Td = inst
    geo = []
    for s in range(N):
        for mm in range(nsurf):
            displace_wing(tr(T, s, mm), vcur[mm], verts_init[mm])
        col, nor, _ = mesh_metrics(0.0, vcur, dtp)
        rv = np.zeros(n, dtp)
        rhs_assemble_velocities(rv, nor, vel_of(Td, s, colloc_h))
        geo.append((col, nor, rv))

    def fmap(xflat):
        x = xflat.reshape(N, n).T  # column-major (n x N)
        te = np.asfortranarray(x[poff[w] + (nc[w] - 1) * ns[w]:poff[w] + nc[w] * ns[w], :])
        R = np.zeros((n, N), dtp, order="F")
        for s in range(N):
            col, nor, rv = geo[s]
            gw = [np.zeros((max_t - 1, a), dtp) for a in ns]
            gamma_wake_from_coeffs(gw[w], te, H, tm[s], omega, dt, int(ts[s]))
            r = rv.copy()
            rhs_assemble_wake_influence(r, gw, col, nor, wake, lifting, int(ts[s]))
            R[:, s] = r
        Y = R @ dft
        Y = lu_solve(lu, piv, Y)
        return np.asarray(Y).T.ravel()

    xs, iters = anderson(np.asarray(x0, dtp).T.ravel() if np.ndim(x0) == 2 else x0, fmap, max_iter, tol, m)
    X = xs.reshape(N, n).T
    fts, ftm, fT, fTd = force_inst
    out = np.zeros((3, N))
    for s in range(N):
        for mm in range(nsurf):
            displace_wing(tr(fT, s, mm), vcur[mm], verts_init[mm])
        col, nor, ar = mesh_metrics(0.0, vcur, dtp)
        vel = vel_of(fTd, s, colloc_h)
        g = X @ dft[s, :]
        dg = X @ ddft[s, :]
        forces = []
        for mm in range(nsurf):
            gm = g[poff[mm]:poff[mm + 1]].reshape(nc[mm], ns[mm])
            dgm = dg[poff[mm]:poff[mm + 1]].reshape(nc[mm], ns[mm])
            d = gamma_delta(gm)
            if coupled_te and mm > 0:
                prev = g[poff[mm - 1]:poff[mm]].reshape(nc[mm - 1], ns[mm - 1])[-1]
                d[0] -= prev
            forces.append(forces_unsteady(vcur[mm], np.ascontiguousarray(d), np.ascontiguousarray(dgm), vel[mm], ar[mm], nor[mm]))
        f_s = np.asarray(fs[s], dtp)
        out[0, s] = coeff_cl_multibody(forces, ar, f_s, 1.0)
        out[1, s] = coeff_cm_multibody(forces, vcur, ar, np.asarray(ref_a[s]), f_s, 1.0)[1]
        if ref_b is not None and nsurf > 1:
            area = asum(ar[1])
            out[2, s] = coeff_cm(forces[1], vcur[1], np.asarray(ref_b[s]), f_s, 1.0, area, mesh_mac(vcur[1], ar[1]))[1]
    return X, out, iters


# ---------------------------------------------------------------------------
# structural integrator (vlm/include/vlm_integrator.hpp:7-41,
# vlm/src/vlm_integrator.cpp:5-68), double
# ---------------------------------------------------------------------------
def newmark_keff(M, C, K, dt, beta=0.25, gamma=0.5):
    """NewmarkBeta::init (vlm_integrator.cpp:5-26): K + M/(beta dt^2) + gamma C/(beta dt)."""
    x1 = gamma / (beta * dt)
    x0 = 1.0 / (beta * dt * dt)
    return np.asarray(K, np.float64) + x0 * np.asarray(M, np.float64) + x1 * np.asarray(C, np.float64)


def newmark_step(M, C, K_eff, v_i, a_i, delta_F, dt, beta=0.25, gamma=0.5):
    """NewmarkBeta::step (vlm_integrator.cpp:28-68): (du, dv, da)."""
    x1 = gamma / (beta * dt)
    x0 = 1.0 / (beta * dt * dt)
    xd0 = 1.0 / (beta * dt)
    xd1 = gamma / beta
    xdd0 = 1.0 / (2.0 * beta)
    xdd1 = -dt * (1.0 - gamma / (2.0 * beta))
    F = np.asarray(delta_F, np.float64) + M @ (xd0 * v_i + xdd0 * a_i) + C @ (xd1 * v_i + xdd1 * a_i)
    du = np.linalg.solve(K_eff, F)
    dv = x1 * du - xd1 * v_i - xdd1 * a_i
    da = x0 * du - xd0 * v_i - xdd0 * a_i
    return du, dv, da


def newmark_linear(M, C, K, u0, v0, dt, steps, beta=0.25, gamma=0.5):
    """Free response of M u'' + C u' + K u = 0 by the incremental steps, as
    the reference's tests/newmark.cpp:108-158 drives them: a_0 from
    M a = -C v_0 - K u_0, then u, v, a += du, dv, da.  Returns (u, v, a),
    each (steps + 1, ndof)."""
    M, C, K = (np.asarray(x, np.float64) for x in (M, C, K))
    n = M.shape[0]
    u = np.zeros((steps + 1, n))
    v = np.zeros((steps + 1, n))
    a = np.zeros((steps + 1, n))
    u[0], v[0] = u0, v0
    a[0] = np.linalg.solve(M, -C @ v[0] - K @ u[0])
    Ke = newmark_keff(M, C, K, dt, beta, gamma)
    for i in range(steps):
        du, dv, da = newmark_step(M, C, Ke, v[i], a[i], np.zeros(n), dt, beta, gamma)
        u[i + 1], v[i + 1], a[i + 1] = u[i] + du, v[i] + dv, a[i] + da
    return u, v, a


# ---------------------------------------------------------------------------
# Coupled aeroelastic 2-DOF (pitch-plunge) UVLM: tests/uvlm_2dof.cpp:437-808
# (COUPLED branch).  Structure in double (Newmark-beta, Newton loop per time
# step on the load increment); aerodynamics in `dtype`.
# ---------------------------------------------------------------------------
def torsional_cubic(alpha, b0=0.0, b1=0.1, b2=0.0, b3=40.0):
    """Cubic pitch stiffness (tests/uvlm_2dof.cpp:238-241)."""
    return b0 + b1 * alpha + b2 * alpha * alpha + b3 * alpha * alpha * alpha


def _rot_y(point_x, angle):
    """rotation_matrix({point_x, 0, 0}, {0, 1, 0}, angle) (vlm_kinematics.hpp:184-201) and d/d(angle)."""
    c, s = math.cos(angle), math.sin(angle)
    R = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    dR = np.array([[-s, 0, c], [0, 0, 0], [-c, 0, -s]])
    p = np.array([point_x, 0.0, 0.0])
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = p - R @ p
    dT = np.zeros((4, 4))
    dT[:3, :3] = dR
    dT[:3, 3] = -dR @ p
    return T, dT


def aero2dof_pose(t_next, h, alpha, hdot, adot, a_h):
    """Dual transform fs(t + dt) . heave . pitch at tau = 0 of the Newton
    iterate (tests/uvlm_2dof.cpp:653-681): value and time derivative (4x4)."""
    Tf = np.eye(4)
    Tf[0, 3] = -t_next
    dTf = np.zeros((4, 4))
    dTf[0, 3] = -1.0
    Th = np.eye(4)
    Th[2, 3] = -h
    dTh = np.zeros((4, 4))
    dTh[2, 3] = -hdot
    Tp, dTp_da = _rot_y(1.0 + a_h, alpha)
    dTp = dTp_da * adot
    T = Tf @ Th @ Tp
    dT = dTf @ Th @ Tp + Tf @ dTh @ Tp + Tf @ Th @ dTp
    return T, dT


def aero2dof_run(verts_init, lifting, vars, t_final, dtype=np.float64, max_iter=50, steps=None, sigma=0.0):
    """UVLM_2DOF::run (tests/uvlm_2dof.cpp:437-808).  verts_init: surfaces in
    dimensional units (quarter-chord shifted), vars: dict of UVLM_2DOF_Vars
    (b, k_a, rho, a_h, omega, zeta_a, zeta_h, x_a, mu, r_a, U_a).  Returns
    dict t, u, v, a, F ((t_steps, 2) each, rows 0 .. last step done), iters
    per step and dt."""
    dt_ = np.dtype(dtype).type
    b = vars["b"]
    vin = []
    for v in verts_init:  # nondimensionalize_verts (:428-435)
        w = np.array(v, np.float64)
        w[:3] /= b
        vin.append(np.ascontiguousarray(w, dtype))
    ns, nc = dims(vin)
    nsurf = len(vin)
    n = sum(x * y for x, y in zip(ns, nc))
    a_h, mu, r_a, Ua, om, rho = vars["a_h"], vars["mu"], vars["r_a"], vars["U_a"], vars["omega"], vars["rho"]
    # initial pose: 3 deg pitch about the elastic axis (:453-467)
    T0, _ = _rot_y(1.0 + a_h, math.radians(3.0))
    verts = [np.empty_like(v) for v in vin]
    for m in range(nsurf):
        displace_wing(np.asfortranarray(T0.astype(dtype)), verts[m], vin[m])
    colloc, normals, areas = mesh_metrics(0.0, verts, dtype)
    colloc_h = [c.copy() for c in colloc]
    # time step = the last chordwise panel's chord of the last surface (:473-480)
    last = vin[-1]
    d = last[:3, -1, 0].astype(np.float32) - last[:3, -2, 0].astype(np.float32)
    dt_nd = float(np.float32(np.sqrt(np.float32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))))
    t_steps = int(np.float32(t_final) / np.float32(dt_nd))
    wake = []
    for s in ns:
        w = np.zeros((4, t_steps, s + 1), dtype)
        w[3] = 1
        wake.append(w)
    gwake = [np.zeros((t_steps - 1, s), dtype) for s in ns]
    # structure (:352-416): K = 0, linear stiffness in the load
    M = np.array([[1.0, vars["x_a"]], [vars["x_a"] / r_a ** 2, 1.0]])
    C = np.array([[2.0 * vars["zeta_h"] * (om / Ua), 0.0], [0.0, 2.0 * vars["zeta_a"] / Ua]])
    K = np.zeros((2, 2))
    Ke = newmark_keff(M, C, K, dt_nd)
    u = np.zeros((t_steps, 2))
    v = np.zeros((t_steps, 2))
    a = np.zeros((t_steps, 2))
    F = np.zeros((t_steps, 2))
    u[0, 1] = math.radians(3.0)
    rhs0 = np.array([-(om / Ua) ** 2 * u[0, 0], -1.0 / (Ua * Ua) * torsional_cubic(u[0, 1])])
    a[0] = np.linalg.solve(M, rhs0 - C @ v[0] - K @ u[0])
    # AIC at the initial pose, no wake, factored once (:504-506)
    lhs = np.zeros((n, n), dtype, order="F")
    lhs_assemble(lhs, colloc, normals, verts, wake, 0, sigma)
    lu, piv = lu_factor(lhs)

    def aero(T, dT, it):
        for m in range(nsurf):
            displace_wing(np.asfortranarray(T.astype(dtype)), verts[m], vin[m])
        col, nor, are = mesh_metrics(0.0, verts, dtype)
        wake_shed(verts, wake, it)
        vel = []
        for m in range(nsurf):
            c = colloc_h[m]
            dd = dT.astype(dtype)
            ve = np.empty_like(c)
            for r in range(3):
                ve[r] = -(dd[r, 0] * c[0] + dd[r, 1] * c[1] + dd[r, 2] * c[2] + dd[r, 3])
            vel.append(ve)
        rhs = np.zeros(n, dtype)
        rhs_assemble_velocities(rhs, nor, vel)
        rhs_assemble_wake_influence(rhs, gwake, col, nor, wake, lifting, it, sigma)
        x = lu_solve(lu, piv, rhs)
        gam, off = [], 0
        for m in range(nsurf):
            gam.append(x[off:off + ns[m] * nc[m]].reshape(nc[m], ns[m]).copy())
            off += ns[m] * nc[m]
        deltas = []
        for m in range(nsurf):
            g = gam[m]
            dl = g.copy()
            gwake[m][t_steps - 2 - it] = g[-1]  # shed the trailing-edge gamma
            if m == 1:  # the reference's wing-flap coupling of the flap's first row (:578-584)
                dl[0] -= gam[0][-1]
            dl[1:] -= g[:-1]
            deltas.append(dl)
        return col, nor, are, vel, gam, deltas

    # t = 0 (:507-515): the initial pose already in place, freestream velocity (1, 0, 0)
    wake_shed(verts, wake, 0)
    vel = []
    for m in range(nsurf):
        c = colloc_h[m]
        ve = np.empty_like(c)
        ve[0], ve[1], ve[2] = dt_(1), dt_(0), dt_(0)
        vel.append(ve)
    rhs = np.zeros(n, dtype)
    rhs_assemble_velocities(rhs, normals, vel)
    x = lu_solve(lu, piv, rhs)
    gam, off = [], 0
    for m in range(nsurf):
        gam.append(x[off:off + ns[m] * nc[m]].reshape(nc[m], ns[m]).copy())
        off += ns[m] * nc[m]
        gwake[m][t_steps - 2] = gam[m][-1]
    nsteps = t_steps - 2 if steps is None else min(steps, t_steps - 2)
    iters = np.zeros(nsteps, np.int32)
    eps = float(np.finfo(np.float32).eps)
    fs = np.array([1.0, 0.0, 0.0], dtype)  # -d/dt of the freestream translation (-t, 0, 0)
    for i in range(nsteps):
        t_nd = float(np.float32(i) * np.float32(dt_nd))
        gprev = [g.copy() for g in gam]
        dF = np.zeros(2)
        du = np.zeros(2)
        du_k = np.ones(2)
        it = 0
        while np.linalg.norm(du_k) > eps:
            du_k = du.copy()
            du, dv, da = newmark_step(M, C, Ke, v[i], a[i], dF, dt_nd)
            u[i + 1], v[i + 1], a[i + 1] = u[i] + du, v[i] + dv, a[i] + da
            T, dT = aero2dof_pose(t_nd + dt_nd, u[i + 1, 0], u[i + 1, 1], v[i + 1, 0], v[i + 1, 1], a_h)
            ref = (T @ np.array([1.0 + a_h, 0.0, 0.0, 1.0]))[:3]
            col, nor, are, vel, gam, deltas = aero(T, dT, i + 1)
            gdts = [((g - gp) * dt_(1.0 / dt_nd)).astype(dtype) for g, gp in zip(gam, gprev)]
            forces = [forces_unsteady(verts[m], deltas[m], gdts[m], vel[m], are[m], nor[m]) for m in range(nsurf)]
            cl = float(coeff_cl_multibody(forces, are, fs, dt_(rho)))
            cm = coeff_cm_multibody(forces, verts, are, ref.astype(dtype), fs, dt_(rho))
            F[i + 1, 0] = -cl / (float(PI_F) * mu)
            F[i + 1, 1] = (2.0 * float(cm[1])) / (float(PI_F) * mu * r_a ** 2)
            dF[0] = F[i + 1, 0] - F[i, 0] - (om / Ua) ** 2 * du[0]
            dF[1] = F[i + 1, 1] - F[i, 1] - 1.0 / (Ua * Ua) * (torsional_cubic(u[i + 1, 1]) - torsional_cubic(u[i, 1]))
            du_k = du_k - du
            it += 1
            if it > max_iter:
                break
        iters[i] = it
    t = np.arange(nsteps + 1) * dt_nd
    return dict(t=t, u=u[:nsteps + 1], v=v[:nsteps + 1], a=a[:nsteps + 1], F=F[:nsteps + 1], iters=iters, dt=dt_nd,
                t_steps=t_steps)


# ---------------------------------------------------------------------------
# Nonlinear VLM (strip-wise viscous correction, van Dam's method)
# ---------------------------------------------------------------------------
def akima_table(x, y, dtype=np.float32):
    """Slopes m (per segment) and spline coefficients s (per point) of
    tiny::AkimaInterpolator (headeronly/tinyinterpolate.hpp:29-54)."""
    T = np.dtype(dtype).type
    x = np.asarray(x, dtype)
    y = np.asarray(y, dtype)
    n = len(x)
    m = np.array([(y[i + 1] - y[i]) / (x[i + 1] - x[i]) for i in range(n - 1)], dtype)
    s = np.zeros(n, dtype)
    s[0] = m[0]
    s[1] = T(0.5) * (m[0] + m[1])
    for i in range(2, n - 2):
        d1 = abs(m[i + 1] - m[i])
        d2 = abs(m[i - 1] - m[i - 2])
        s[i] = (d1 * m[i - 1] + d2 * m[i]) / (d1 + d2) if d1 + d2 > T(0) else T(0.5) * (m[i] + m[i - 1])
    s[n - 2] = T(0.5) * (m[n - 3] + m[n - 2])
    s[n - 1] = m[n - 2]
    return x, y, m, s


def akima_eval(tab, xq):
    """tiny::AkimaInterpolator::operator() (tinyinterpolate.hpp:56-73):
    cubic on the interval holding xq (std::lower_bound), linear with the end
    segment's slope outside the table."""
    x, y, m, s = tab
    T = x.dtype.type
    xq = T(xq)
    idx = int(np.searchsorted(x, xq, side="left"))
    if idx == 0:
        return T(y[0] - m[0] * (x[0] - xq))
    if idx == len(x):
        return T(y[-1] + m[-1] * (xq - x[-1]))
    i = idx - 1
    dx = x[i + 1] - x[i]
    dxx = xq - x[i]
    a, b = y[i], s[i]
    c = (T(3) * m[i] - T(2) * s[i] - s[i + 1]) / dx
    d = (s[i] + s[i + 1] - T(2) * m[i]) / (dx * dx)
    return T(a + b * dxx + c * dxx * dxx + d * dxx * dxx * dxx)


def nlvlm_run(verts_init, alpha, db_alpha, db_cl, beta=0.0, u_inf=1.0, rho=1.0, dtype=np.float32, tol=1e-5,
              max_iter=100):
    """NLVLM::run (vlm/src/vlm.cpp:198-295, defaults vlm.hpp:90-91).

    The wing and its single 100-chord wake row as in VLM::run, one AIC
    factored once.  Each iteration: panel velocities from the strip angles
    (vlm.cpp:186-196: beta = 0 there), RHS, solve, gamma deltas, steady
    forces; per spanwise strip its CL about the strip's own lift axis, the
    effective angle CL/(2 pi) - alpha_strip + alpha, and the correction
    (CL_polar(effective) - CL)/(2 pi) added to the strip angle; the L1 sum of
    the corrections divided by the panel count ends the loop below `tol`.
    The final CL resets the strip angles to alpha (:281-285) and is
    coeff_cl_multibody of the last circulation.  The polar is the Akima
    interpolant of (db_alpha, db_cl) (Database2D::interpolate_CL,
    vlm_data.hpp:85-90: the first profile, no blending in y).

    Returns dict(cl, iters, err, strip_alpha (list per surface, before the
    reset), gamma)."""
    T = np.dtype(dtype).type
    tab = akima_table(db_alpha, db_cl, dtype)
    verts_init = [np.ascontiguousarray(v, dtype) for v in verts_init]
    verts = [v.copy() for v in verts_init]
    ns, nc = dims(verts)
    n = sum(a * b for a, b in zip(ns, nc))
    wake = []
    for s in ns:
        w = np.zeros((4, 2, s + 1), dtype)
        w[3] = 1
        wake.append(w)
    a32 = T(alpha)
    tr = translation(np.array([T(-100.0) * T(u_inf) * np.cos(a32), T(0), T(-100.0) * T(u_inf) * np.sin(a32)], dtype),
                     dtype)
    wake_shed(verts, wake, 0)
    for v, vi in zip(verts, verts_init):
        displace_wing(tr, v, vi)
    wake_shed(verts, wake, 1)
    colloc, normals, areas = mesh_metrics(alpha, verts, dtype)
    lhs = np.zeros((n, n), dtype, order="F")
    lhs_assemble(lhs, colloc, normals, verts, wake, 1, 0.0)
    lu, piv = lu_factor(lhs)
    strips = [np.full(s, a32, dtype) for s in ns]
    two_pi = T(np.float32(2.0) * np.float32(3.141593))  # 2 PI_f, the reference's float pi (vlm_types.hpp:22)

    def velocities():
        out = []
        for st, s, c in zip(strips, ns, nc):
            v = np.empty((3, c, s), dtype)
            for i in range(s):
                f = freestream(u_inf, st[i], 0.0, dtype)
                v[:, :, i] = f[:, None]
            out.append(v)
        return out

    err, it = 1.0, 0
    deltas, gam = None, None
    while it < max_iter and err > tol:
        err = 0.0
        vel = velocities()
        rhs = np.zeros(n, dtype)
        rhs_assemble_velocities(rhs, normals, vel)
        x = lu_solve(lu, piv, rhs)
        gam, deltas = [], []
        off = 0
        for s, c in zip(ns, nc):
            g = x[off:off + s * c].reshape(c, s).copy()
            off += s * c
            gam.append(g)
            deltas.append(gamma_delta(g))
        forces = [forces_steady(v, d, u) for v, d, u in zip(verts, deltas, vel)]
        for st, f, a in zip(strips, forces, areas):
            for i in range(len(st)):
                fi = np.ascontiguousarray(f[:, :, i:i + 1])
                area = asum(np.ascontiguousarray(a[:, i:i + 1]))
                fs_i = freestream(u_inf, st[i], beta, dtype)
                cl_i = coeff_cl(fi, lift_axis(fs_i), fs_i, T(rho), area)
                eff = T(cl_i / two_pi - st[i] + a32)
                corr = T((akima_eval(tab, eff) - cl_i) / two_pi)
                st[i] = T(st[i] + corr)
                err += abs(float(corr))
        err /= float(n)
        it += 1
    strip_out = [st.copy() for st in strips]
    for st in strips:
        st[:] = a32
    vel = velocities()
    forces = [forces_steady(v, d, u) for v, d, u in zip(verts, deltas, vel)]
    fs = freestream(u_inf, alpha, beta, dtype)
    cl = coeff_cl_multibody(forces, areas, fs, T(rho))
    return dict(cl=cl, iters=it, err=err, strip_alpha=strip_out, gamma=gam)
