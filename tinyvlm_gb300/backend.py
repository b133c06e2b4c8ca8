"""Python mirror of the tinyvlm plugin API (``vlm::Backend``, ``vlm::LU``,
``vlm::BLAS``, ``vlm::LSQ``, ``vlm::Memory``) over the gbvlm C ABI.

Method names, argument order and meaning follow
vlm/include/vlm_backend.hpp:13-136 and vlm/include/vlm_memory.hpp:22-37.
Arguments are device arrays -- ``tinyvlm_gb300.device.DeviceArray``, or any
object with ``data_ptr()``, ``shape``, ``dtype`` and ``is_cuda`` -- laid out
like the reference tensors:

  wing vertices  (4, nc+1, ns+1)  == reference (ns+1, nc+1, 4)
  panel vectors  (3, nc, ns)      == reference (ns, nc, 3)
  panel scalars  (nc, ns)         == reference (ns, nc)
  wake vertices  (4, nwv, ns+1)   == reference (ns+1, nwv, 4)
  wake gamma     (nwv-1, ns)      == reference (ns, nwv-1)
  LHS            (n, n) holding the column-major matrix, i.e. lhs[col, row]

Multi-surface arguments are Python lists (the reference's MultiTensorView).
Errors raise ``GbvlmError`` instead of the reference's print-and-exit.  No
other CUDA binding is needed: device memory, streams and events come from
the library itself (device.py).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import F32, F64, call, dims_array, ptr_array
from .device import DeviceArray, dtype_name, stream_handle

__all__ = ["Backend", "LU", "BLAS", "LSQ", "Memory", "create_backend", "get_available_backends"]


def _check(t, dtype, name):
    if not getattr(t, "is_cuda", False) or not hasattr(t, "data_ptr"):
        raise TypeError("%s must be a device array" % name)
    if dtype_name(t.dtype) != dtype:
        raise TypeError("%s has dtype %s, expected %s" % (name, dtype_name(t.dtype), dtype))
    if hasattr(t, "is_contiguous") and not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    return t.data_ptr()


def _ndim(t):
    return len(t.shape)


def _numel(t):
    return int(np.prod(t.shape, dtype=np.int64))


class Backend:
    """GB300 backend: every operator runs as a hand-written sm_103a kernel."""

    name = "gb300"

    def __init__(self, dtype=np.float32, stream=None):
        name = dtype_name(dtype)
        if name not in ("float32", "float64"):
            raise ValueError("dtype must be float32 or float64")
        self.dtype = name
        self.np_dtype = np.dtype(name)
        self.sfx = "f32" if name == "float32" else "f64"
        self.R = F32 if name == "float32" else F64
        self.sigma_vatistas = 0.0
        self._stream = stream
        self.memory = Memory(self)
        self.blas = BLAS(self)

    # -- helpers -----------------------------------------------------------
    def stream(self):
        """The stream every call runs on: the one given at construction, else the legacy default stream."""
        return stream_handle(self._stream)

    def _ptrs(self, ts, name):
        return ptr_array([_check(t, self.dtype, name) for t in ts])

    @staticmethod
    def _dims_from_verts(verts_wing, verts_wake=None):
        d = []
        for m, v in enumerate(verts_wing):
            nwv = verts_wake[m].shape[1] if verts_wake is not None else 0
            d.append((v.shape[2] - 1, v.shape[1] - 1, nwv))
        return dims_array(d)

    @staticmethod
    def _dims_from_panels(panels, verts_wake=None):
        d = []
        for m, p in enumerate(panels):
            nwv = verts_wake[m].shape[1] if verts_wake is not None else 0
            d.append((p.shape[-1], p.shape[-2], nwv))
        return dims_array(d)

    # -- vlm::Backend pure virtuals -----------------------------------------
    def lhs_assemble(self, lhs, colloc, normals, verts_wing, verts_wake, iteration):
        d = self._dims_from_verts(verts_wing, verts_wake if verts_wake is not None else None)
        c, _k1 = self._ptrs(colloc, "colloc")
        n, _k2 = self._ptrs(normals, "normals")
        vw, _k3 = self._ptrs(verts_wing, "verts_wing")
        if verts_wake is not None:
            vk, _k4 = self._ptrs(verts_wake, "verts_wake")
        else:
            vk, _k4 = None, None
        call("gbvlm_lhs_assemble_" + self.sfx, _check(lhs, self.dtype, "lhs"), lhs.shape[1], len(verts_wing), d,
             c, n, vw, vk, int(iteration), self.R(self.sigma_vatistas), self.stream())

    def rhs_assemble_velocities(self, rhs, normals, velocities):
        d = self._dims_from_panels(normals)
        n, _k1 = self._ptrs(normals, "normals")
        v, _k2 = self._ptrs(velocities, "velocities")
        call("gbvlm_rhs_assemble_velocities_" + self.sfx, _check(rhs, self.dtype, "rhs"), len(normals), d, n, v,
             self.stream())

    def rhs_assemble_wake_influence(self, rhs, gamma_wake, colloc, normals, verts_wake, lifting, iteration):
        d = self._dims_from_panels(normals, verts_wake)
        g, _k1 = self._ptrs(gamma_wake, "gamma_wake")
        c, _k2 = self._ptrs(colloc, "colloc")
        n, _k3 = self._ptrs(normals, "normals")
        vk, _k4 = self._ptrs(verts_wake, "verts_wake")
        lf = (ctypes.c_int32 * len(lifting))(*[1 if x else 0 for x in lifting])
        call("gbvlm_rhs_assemble_wake_influence_" + self.sfx, _check(rhs, self.dtype, "rhs"), len(normals), d, g, c,
             n, vk, ctypes.cast(lf, ctypes.c_void_p), int(iteration), self.R(self.sigma_vatistas), self.stream())

    def forces_steady(self, verts_wing, gamma_delta, velocities, forces):
        nc, ns = gamma_delta.shape
        call("gbvlm_forces_steady_" + self.sfx, ns, nc, _check(verts_wing, self.dtype, "verts_wing"),
             _check(gamma_delta, self.dtype, "gamma_delta"), _check(velocities, self.dtype, "velocities"),
             _check(forces, self.dtype, "forces"), self.stream())

    def forces_unsteady(self, verts_wing, gamma_delta, dgamma_dt, velocities, areas, normals, forces):
        nc, ns = gamma_delta.shape
        call("gbvlm_forces_unsteady_" + self.sfx, ns, nc, _check(verts_wing, self.dtype, "verts_wing"),
             _check(gamma_delta, self.dtype, "gamma_delta"), _check(dgamma_dt, self.dtype, "dgamma_dt"),
             _check(velocities, self.dtype, "velocities"), _check(areas, self.dtype, "areas"),
             _check(normals, self.dtype, "normals"), _check(forces, self.dtype, "forces"), self.stream())

    def _ctype(self):
        return ctypes.c_float if self.sfx == "f32" else ctypes.c_double

    def _vec(self, v):
        return (self._ctype() * 3)(*[float(x) for x in v])

    def coeff_cl(self, forces, lift_axis, freestream, rho, area):
        _, nc, ns = forces.shape
        T = self._ctype()
        out = T()
        la, fs = self._vec(lift_axis), self._vec(freestream)
        call("gbvlm_coeff_cl_" + self.sfx, ns, nc, _check(forces, self.dtype, "forces"),
             ctypes.cast(la, ctypes.c_void_p), ctypes.cast(fs, ctypes.c_void_p), self.R(rho), self.R(area),
             ctypes.cast(ctypes.pointer(out), ctypes.c_void_p), self.stream())
        return out.value

    def coeff_cm(self, forces, verts_wing, ref_pt, freestream, rho, area, mac):
        _, nc, ns = forces.shape
        T = self._ctype()
        out = (T * 3)()
        rp, fs = self._vec(ref_pt), self._vec(freestream)
        call("gbvlm_coeff_cm_" + self.sfx, ns, nc, _check(forces, self.dtype, "forces"),
             _check(verts_wing, self.dtype, "verts_wing"), ctypes.cast(rp, ctypes.c_void_p),
             ctypes.cast(fs, ctypes.c_void_p), self.R(rho), self.R(area), self.R(mac),
             ctypes.cast(out, ctypes.c_void_p), self.stream())
        return tuple(out)

    def mesh_metrics(self, alpha_rad, verts_wing, colloc, normals, areas):
        d = self._dims_from_verts(verts_wing)
        v, _k1 = self._ptrs(verts_wing, "verts_wing")
        c, _k2 = self._ptrs(colloc, "colloc")
        n, _k3 = self._ptrs(normals, "normals")
        a, _k4 = self._ptrs(areas, "areas")
        call("gbvlm_mesh_metrics_" + self.sfx, self.R(alpha_rad), len(verts_wing), d, v, c, n, a, self.stream())

    def mesh_mac(self, verts_wing, areas):
        nc, ns = areas.shape
        T = self._ctype()
        out = T()
        call("gbvlm_mesh_mac_" + self.sfx, ns, nc, _check(verts_wing, self.dtype, "verts_wing"),
             _check(areas, self.dtype, "areas"), ctypes.cast(ctypes.pointer(out), ctypes.c_void_p), self.stream())
        return out.value

    def gamma_wake_from_coeffs(self, gamma_wake, gamma_coeffs, harmonics, tn, omega, dt, iteration):
        ncols, ns = gamma_wake.shape
        call("gbvlm_gamma_wake_from_coeffs_" + self.sfx, _check(gamma_wake, self.dtype, "gamma_wake"), ns, ncols,
             _check(gamma_coeffs, self.dtype, "gamma_coeffs"), int(harmonics), self.R(tn), self.R(omega),
             self.R(dt), int(iteration), self.stream())

    def sum(self, tensor, shape=None, strides=None):
        """Backend::sum.  A 1-D array sums its entries (sum(TV1f&)); a 2-D
        view (sum(TV2f&), vlm_backend_cpu.cpp:515-523) is given by ``shape``
        = (m, n) and element ``strides`` = (s0, s1) over the array's memory,
        in the reference's index order; a 2-D array without them is summed
        whole."""
        T = self._ctype()
        out = T()
        ptr = _check(tensor, self.dtype, "tensor")
        if shape is None and _ndim(tensor) < 2:
            call("gbvlm_sum_" + self.sfx, ptr, _numel(tensor), ctypes.cast(ctypes.pointer(out), ctypes.c_void_p),
                 self.stream())
            return out.value
        if shape is None:
            m = int(tensor.shape[-1])
            shape, strides = (m, _numel(tensor) // m), (1, m)
        call("gbvlm_sum2d_" + self.sfx, ptr, int(shape[0]), int(shape[1]), int(strides[0]), int(strides[1]),
             ctypes.cast(ctypes.pointer(out), ctypes.c_void_p), self.stream())
        return out.value

    # -- non-virtual multibody helpers (vlm_backend.hpp:58-71) --------------
    def displace_wing(self, transforms, verts_wing, verts_wing_init):
        d = self._dims_from_verts(verts_wing)
        t, _k1 = self._ptrs(transforms, "transforms")
        v, _k2 = self._ptrs(verts_wing, "verts_wing")
        vi, _k3 = self._ptrs(verts_wing_init, "verts_wing_init")
        call("gbvlm_displace_wing_" + self.sfx, len(verts_wing), d, t, v, vi, self.stream())

    def wake_shed(self, verts_wing, verts_wake, iteration):
        d = self._dims_from_verts(verts_wing, verts_wake)
        v, _k1 = self._ptrs(verts_wing, "verts_wing")
        k, _k2 = self._ptrs(verts_wake, "verts_wake")
        call("gbvlm_wake_shed_" + self.sfx, len(verts_wing), d, v, k, int(iteration), self.stream())

    def wake_rollup(self, verts_wake, verts_wing, gamma_wing, gamma_wake, lifting, dt, iteration):
        """Free-wake roll-up (the reference's dead kernel_rollup, given a caller)."""
        d = self._dims_from_verts(verts_wing, verts_wake)
        k, _k1 = self._ptrs(verts_wake, "verts_wake")
        v, _k2 = self._ptrs(verts_wing, "verts_wing")
        g, _k3 = self._ptrs(gamma_wing, "gamma_wing")
        gw, _k4 = self._ptrs(gamma_wake, "gamma_wake")
        lf = (ctypes.c_int32 * len(lifting))(*[1 if x else 0 for x in lifting])
        call("gbvlm_wake_rollup_" + self.sfx, len(verts_wing), d, k, v, g, gw, ctypes.cast(lf, ctypes.c_void_p),
             self.R(self.sigma_vatistas), self.R(dt), int(iteration), self.stream())

    def trefftz_cd(self, verts_wake, gamma_wake, freestream, area):
        _, nwv, n = verts_wake.shape
        T = self._ctype()
        out = T()
        fs = self._vec(freestream)
        call("gbvlm_trefftz_cd_" + self.sfx, n - 1, nwv, _check(verts_wake, self.dtype, "verts_wake"),
             _check(gamma_wake, self.dtype, "gamma_wake"), ctypes.cast(fs, ctypes.c_void_p), self.R(area),
             self.R(self.sigma_vatistas), ctypes.cast(ctypes.pointer(out), ctypes.c_void_p), self.stream())
        return out.value

    def gamma_update(self, x, gamma, gamma_delta, gamma_wake=None, wake_col=0, gamma_prev=None, dgamma_dt=None,
                     dt=0.0):
        nc, ns = gamma.shape
        call("gbvlm_gamma_update_" + self.sfx, ns, nc, _check(x, self.dtype, "x"), _check(gamma, self.dtype, "gamma"),
             _check(gamma_delta, self.dtype, "gamma_delta"),
             None if gamma_wake is None else _check(gamma_wake, self.dtype, "gamma_wake"), int(wake_col),
             None if gamma_prev is None else _check(gamma_prev, self.dtype, "gamma_prev"),
             None if dgamma_dt is None else _check(dgamma_dt, self.dtype, "dgamma_dt"), self.R(dt), self.stream())

    # -- factories (vlm_backend.hpp:72-75) -----------------------------------
    def create_lu_solver(self):
        return LU(self)

    def create_memory_manager(self):
        return Memory(self)

    def create_blas(self):
        return BLAS(self)

    def create_lsq_solver(self):
        return LSQ(self)


class LU:
    """vlm::LU (vlm_backend.hpp:99-119): init / factorize / solve."""

    def __init__(self, backend):
        self.backend = backend
        h = ctypes.c_void_p()
        call("gbvlm_lu_create", ctypes.cast(ctypes.pointer(h), ctypes.c_void_p))
        self.h = h

    def __del__(self):
        try:
            if self.h:
                _lib.lib().gbvlm_lu_destroy(self.h)
        except Exception:
            pass

    def init(self, A):
        call("gbvlm_lu_init", self.h, A.shape[0])

    def factorize(self, A):
        b = self.backend
        call("gbvlm_lu_factor_" + b.sfx, self.h, _check(A, b.dtype, "A"), A.shape[0], A.shape[1], b.stream())

    def solve(self, A, x):
        b = self.backend
        nrhs = 1 if _ndim(x) == 1 else x.shape[0]
        n = A.shape[0]
        call("gbvlm_lu_solve_" + b.sfx, self.h, _check(A, b.dtype, "A"), n, A.shape[1], _check(x, b.dtype, "x"),
             n, nrhs, b.stream())


class Memory:
    """vlm::Memory (vlm_memory.hpp:22-37): device memory from cudaMalloc, host
    memory pinned.  Pointers are plain integers."""

    DEVICE, HOST = 0, 1

    def __init__(self, backend):
        self.backend = backend

    def alloc(self, location, size_bytes):
        p = ctypes.c_void_p()
        call("gbvlm_mem_alloc", int(location), int(size_bytes), ctypes.cast(ctypes.pointer(p), ctypes.c_void_p))
        return p.value or 0

    def free(self, location, ptr):
        call("gbvlm_mem_free", int(location), ctypes.c_void_p(ptr))

    def copy(self, dst_loc, dst, dst_stride, src_loc, src, src_stride, elem_size, size):
        call("gbvlm_mem_copy", int(dst_loc), ctypes.c_void_p(dst), int(dst_stride), int(src_loc),
             ctypes.c_void_p(src), int(src_stride), int(elem_size), int(size), self.backend.stream())

    def fill(self, location, ptr, stride, value, size):
        call("gbvlm_mem_fill_" + self.backend.sfx, int(location), ctypes.c_void_p(ptr), int(stride),
             self.backend.R(value), int(size), self.backend.stream())


class BLAS:
    """vlm::BLAS (vlm_backend.hpp:78-97) on the backend's precision.  Matrices
    are the reference's column-major 2-D views: a C-ordered (cols, rows)
    array holds a rows x cols matrix with leading dimension rows."""

    NO, YES = 0, 1

    def __init__(self, backend):
        self.b = backend

    def _m(self, A, name):
        """(rows, cols, ld, ptr) of a C-ordered (cols, rows) array."""
        return int(A.shape[-1]), _numel(A) // int(A.shape[-1]), int(A.shape[-1]), _check(A, self.b.dtype, name)

    def gemv(self, alpha, A, x, beta, y, trans=0):
        m, n, lda, pa = self._m(A, "A")
        call("gbvlm_blas_gemv_" + self.b.sfx, int(bool(trans)), m, n, self.b.R(alpha), pa, lda,
             _check(x, self.b.dtype, "x"), 1, self.b.R(beta), _check(y, self.b.dtype, "y"), 1, self.b.stream())

    def gemm(self, alpha, A, B, beta, C, trans_a=0, trans_b=0):
        ra, ca, lda, pa = self._m(A, "A")
        rb, cb, ldb, pb = self._m(B, "B")
        m, n, ldc, pc = self._m(C, "C")
        k = ra if trans_a else ca
        if (ca if trans_a else ra) != m or (rb if trans_b else cb) != n or (cb if trans_b else rb) != k:
            raise ValueError("gemm: shapes do not agree")
        call("gbvlm_blas_gemm_" + self.b.sfx, int(bool(trans_a)), int(bool(trans_b)), m, n, k, self.b.R(alpha), pa,
             lda, pb, ldb, self.b.R(beta), pc, ldc, self.b.stream())

    def axpy(self, alpha, x, y):
        """y += alpha x over whole arrays of the same size (the 1-D and the 2-D overloads alike)."""
        if _numel(x) != _numel(y):
            raise ValueError("axpy: sizes differ")
        call("gbvlm_blas_axpy_" + self.b.sfx, _numel(x), self.b.R(alpha), _check(x, self.b.dtype, "x"), 1,
             _check(y, self.b.dtype, "y"), 1, self.b.stream())

    def axpy_strided(self, alpha, x, x_view, y, y_view):
        """BLAS::axpy(TV2f, TV2f): views given as (offset, m, n, s0, s1) element tuples over x and y."""
        item = self.b.np_dtype.itemsize
        xo, m, n, xs0, xs1 = x_view
        yo, ym, yn, ys0, ys1 = y_view
        if (m, n) != (ym, yn):
            raise ValueError("axpy: view shapes differ")
        call("gbvlm_blas_axpy2d_" + self.b.sfx, int(m), int(n), self.b.R(alpha),
             ctypes.c_void_p(_check(x, self.b.dtype, "x") + item * int(xo)), int(xs0), int(xs1),
             ctypes.c_void_p(_check(y, self.b.dtype, "y") + item * int(yo)), int(ys0), int(ys1), self.b.stream())

    def scal(self, alpha, x):
        call("gbvlm_blas_scal_" + self.b.sfx, _numel(x), self.b.R(alpha), _check(x, self.b.dtype, "x"), 1,
             self.b.stream())

    def norm(self, x):
        out = self.b._ctype()()
        call("gbvlm_blas_nrm2_" + self.b.sfx, _numel(x), _check(x, self.b.dtype, "x"), 1,
             ctypes.cast(ctypes.pointer(out), ctypes.c_void_p), self.b.stream())
        return out.value


class LSQ:
    """vlm::LSQ (vlm_backend.hpp:121-133): least squares min ||A x - B|| by
    Householder QR; ``solve`` leaves x in the first n rows of B (LAPACK ?gels
    semantics).  A: C-ordered (n, m) array holding the m x n column-major
    matrix; B: (nrhs, m)."""

    def __init__(self, backend):
        self.b = backend

    def init(self, A, B):
        pass  # no workspace to size

    def solve(self, A, B):
        m = int(A.shape[-1])
        n = _numel(A) // m
        nrhs = _numel(B) // m
        if int(B.shape[-1]) != m:
            raise ValueError("LSQ: B must have m = %d rows" % m)
        call("gbvlm_lsq_solve_" + self.b.sfx, m, n, _check(A, self.b.dtype, "A"), m, _check(B, self.b.dtype, "B"),
             nrhs, m, self.b.stream())


def get_available_backends():
    return ["gb300"]


def create_backend(name, dtype=np.float32):
    """create_backend (vlm/src/vlm_backend.cpp:15-27): "gb300"; "cuda" and
    "cpu", the names the reference's scripts pass, select it too."""
    if name not in ("gb300", "cuda", "cpu"):
        raise RuntimeError("Unsupported backend: " + name)
    return Backend(dtype)
