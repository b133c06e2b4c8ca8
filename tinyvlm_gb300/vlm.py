"""Simulation drivers (vlm/include/vlm.hpp) over the gbvlm C ABI.

``VLM(backend_name, meshes).run(FlowData)`` mirrors vlm/src/vlm.cpp:17-151
and ``NLVLM(backend_name, meshes).run(FlowData, Database)`` vlm.cpp:153-295:
meshes are plot3d paths (read with the quarter-chord shift, like
``Simulation``) or ``(4, nc+1, ns+1)`` vertex arrays already shifted.
"""
import ctypes
import math

import numpy as np

from . import _lib
from ._lib import Coeffs, call, dims_array
from .device import stream_handle

__all__ = ["FlowData", "AeroCoefficients", "VLM", "NLVLM", "WingProfile", "Database", "read_plot3d"]


class FlowData:
    """vlm/include/vlm_data.hpp:11-25 with vlm/src/vlm_utils.cpp:5-19."""

    def __init__(self, alpha, beta=0.0, u_inf=1.0, rho=1.0):
        self.alpha, self.beta, self.u_inf, self.rho = float(alpha), float(beta), float(u_inf), float(rho)
        ca, sa, cb, sb = math.cos(alpha), math.sin(alpha), math.cos(beta), math.sin(beta)
        self.freestream = np.array([u_inf * ca * cb, -u_inf * ca * sb, u_inf * sa])
        la = np.array([-self.freestream[2], 0.0, self.freestream[0]])
        self.lift_axis = la / np.linalg.norm(la)
        self.stream_axis = self.freestream / np.linalg.norm(self.freestream)


class AeroCoefficients:
    def __init__(self, cl, cd, cm):
        self.cl, self.cd, self.cm = cl, cd, cm

    def __repr__(self):
        return "AeroCoefficients(cl=%.8g, cd=%.8g, cm=%s)" % (self.cl, self.cd, list(self.cm))


def read_plot3d(path, qc=True):
    """plot3d reader of the C ABI (vlm/src/vlm_mesh.cpp); returns (4, nc+1, ns+1) float32."""
    d = _lib.Dims()
    call("gbvlm_read_plot3d", path.encode(), 1 if qc else 0, ctypes.cast(ctypes.pointer(d), ctypes.c_void_p), None)
    v = np.zeros((4, d.nc + 1, d.ns + 1), np.float32)
    call("gbvlm_read_plot3d", path.encode(), 1 if qc else 0, ctypes.cast(ctypes.pointer(d), ctypes.c_void_p),
         ctypes.c_void_p(v.ctypes.data))
    return v


class VLM:
    """Steady VLM on the GPU.  ``precision=32`` keeps the reference's float
    semantics; ``precision=64`` is the plain per-solve double path."""

    def __init__(self, backend_name, meshes, precision=32):
        if backend_name not in ("gb300", "cuda", "cpu"):
            raise RuntimeError("Unsupported backend: " + backend_name)
        verts = [read_plot3d(m) if isinstance(m, str) else np.ascontiguousarray(m, np.float32) for m in meshes]
        self.verts = verts
        self.dims = [(v.shape[2] - 1, v.shape[1] - 1, 0) for v in verts]
        self.n = sum(a * b for a, b, _ in self.dims)
        d = dims_array(self.dims)
        arr = (ctypes.c_void_p * len(verts))(*[v.ctypes.data for v in verts])
        h = ctypes.c_void_p()
        call("gbvlm_vlm_create", ctypes.cast(ctypes.pointer(h), ctypes.c_void_p), len(verts), d,
             ctypes.cast(arr, _lib.PP), int(precision))
        self.h = h

    def __del__(self):
        try:
            if self.h:
                _lib.lib().gbvlm_vlm_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def run(self, flow, ref_pt=(0.0, 0.0, 0.0), return_gamma=False, stream=None):
        out = Coeffs()
        rp = (ctypes.c_double * 3)(*ref_pt)
        g = np.zeros(self.n, np.float64) if return_gamma else None
        s = stream_handle(stream)
        call("gbvlm_vlm_run", self.h, flow.alpha, flow.beta, flow.u_inf, flow.rho, ctypes.cast(rp, ctypes.c_void_p),
             ctypes.cast(ctypes.pointer(out), ctypes.c_void_p),
             ctypes.c_void_p(g.ctypes.data) if g is not None else None, s)
        res = AeroCoefficients(out.cl, out.cdi, tuple(out.cm))
        if return_gamma:
            return res, g
        return res

    def run_shared(self, alphas, u_inf=1.0, rho=1.0, ref_pt=(0.0, 0.0, 0.0), return_gamma=False, stream=None):
        """One AIC at alpha = 0 factored once, every angle a right-hand side (the
        classical linear sweep of the large steady workload), on this
        handle's precision; returns one AeroCoefficients per angle."""
        al = np.ascontiguousarray(alphas, np.float64)
        out = (Coeffs * len(al))()
        rp = (ctypes.c_double * 3)(*ref_pt)
        g = np.zeros((len(al), self.n), np.float64) if return_gamma else None
        s = stream_handle(stream)
        call("gbvlm_vlm_run_shared", self.h, len(al), ctypes.c_void_p(al.ctypes.data), float(u_inf), float(rho),
             ctypes.cast(rp, ctypes.c_void_p), ctypes.cast(out, ctypes.c_void_p),
             ctypes.c_void_p(g.ctypes.data) if g is not None else None, s)
        res = [AeroCoefficients(o.cl, o.cdi, tuple(o.cm)) for o in out]
        if return_gamma:
            return res, g
        return res


class WingProfile:
    """A 2D section polar (vlm/include/vlm_data.hpp:40-77): coefficients
    against the angle of attack (radians).  NLVLM uses the lift curve."""

    def __init__(self, alphas, CL, CD=None, CMx=None, CMy=None, CMz=None):
        self.alphas = np.ascontiguousarray(alphas, np.float32)
        self.CL = np.ascontiguousarray(CL, np.float32)
        z = np.zeros_like(self.alphas)
        self.CD, self.CMx, self.CMy, self.CMz = [z if c is None else np.ascontiguousarray(c, np.float32)
                                                 for c in (CD, CMx, CMy, CMz)]
        if self.alphas.shape != self.CL.shape or len(self.alphas) < 4:
            raise ValueError("a profile needs at least 4 (alpha, CL) points of the same length")


class Database:
    """Database2D (vlm_data.hpp:79-91): profiles at spanwise positions; like
    the reference, interpolation uses the first profile only."""

    def __init__(self):
        self.profiles = []
        self.profiles_pos = []


class NLVLM:
    """Nonlinear VLM on the GPU (vlm/src/vlm.cpp:153-295): strip angles
    corrected toward the database's lift polar until the L1 correction per
    panel falls below ``tol`` (reference defaults: tol 1e-5, 100
    iterations).  ``run`` returns AeroCoefficients(cl, 0, 0) as the reference
    does; ``iters``, ``err`` and ``strip_alpha`` (per surface, before the
    final reset to alpha) describe the last run."""

    DEFAULT_TOL = 1e-5
    DEFAULT_MAX_ITER = 100

    def __init__(self, backend_name, meshes, precision=32):
        if backend_name not in ("gb300", "cuda", "cpu"):
            raise RuntimeError("Unsupported backend: " + backend_name)
        verts = [read_plot3d(m) if isinstance(m, str) else np.ascontiguousarray(m, np.float32) for m in meshes]
        self.verts = verts
        self.dims = [(v.shape[2] - 1, v.shape[1] - 1, 0) for v in verts]
        d = dims_array(self.dims)
        arr = (ctypes.c_void_p * len(verts))(*[v.ctypes.data for v in verts])
        h = ctypes.c_void_p()
        call("gbvlm_nlvlm_create", ctypes.cast(ctypes.pointer(h), ctypes.c_void_p), len(verts), d,
             ctypes.cast(arr, _lib.PP), int(precision))
        self.h = h
        self.max_iter, self.tol = self.DEFAULT_MAX_ITER, self.DEFAULT_TOL
        self.iters, self.err, self.strip_alpha = 0, None, None

    def __del__(self):
        try:
            if self.h:
                _lib.lib().gbvlm_nlvlm_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def run(self, flow, db, stream=None):
        prof = db.profiles[0]
        cl = ctypes.c_double()
        it = ctypes.c_int32()
        err = ctypes.c_double()
        strips = np.zeros(sum(ns for ns, _, _ in self.dims), np.float32)
        s = stream_handle(stream)
        call("gbvlm_nlvlm_run", self.h, flow.alpha, flow.beta, flow.u_inf, flow.rho,
             ctypes.c_void_p(prof.alphas.ctypes.data), ctypes.c_void_p(prof.CL.ctypes.data), len(prof.alphas),
             float(self.tol), int(self.max_iter), ctypes.cast(ctypes.pointer(cl), ctypes.c_void_p),
             ctypes.cast(ctypes.pointer(it), ctypes.c_void_p), ctypes.cast(ctypes.pointer(err), ctypes.c_void_p),
             ctypes.c_void_p(strips.ctypes.data), s)
        self.iters, self.err = it.value, err.value
        self.strip_alpha, o = [], 0
        for ns, _, _ in self.dims:
            self.strip_alpha.append(strips[o:o + ns].copy())
            o += ns
        return AeroCoefficients(cl.value, 0.0, (0.0, 0.0, 0.0))
