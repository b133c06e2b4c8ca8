"""Python mirror of the tinyvlm plugin API (``vlm::Backend``, ``vlm::LU``)
over the gbvlm C ABI.

Method names, argument order and meaning follow
vlm/include/vlm_backend.hpp:13-136.  Arguments are CUDA ``torch`` tensors
(torch only provides device memory and the stream) laid out like the
reference tensors:

  wing vertices  (4, nc+1, ns+1)  == reference (ns+1, nc+1, 4)
  panel vectors  (3, nc, ns)      == reference (ns, nc, 3)
  panel scalars  (nc, ns)         == reference (ns, nc)
  wake vertices  (4, nwv, ns+1)   == reference (ns+1, nwv, 4)
  wake gamma     (nwv-1, ns)      == reference (ns, nwv-1)
  LHS            (n, n) holding the column-major matrix, i.e. lhs[col, row]

Multi-surface arguments are Python lists (the reference's MultiTensorView).
Errors raise ``GbvlmError`` instead of the reference's print-and-exit.
"""
import ctypes

import torch

from . import _lib
from ._lib import F32, F64, call, dims_array, ptr_array

__all__ = ["Backend", "LU", "create_backend", "get_available_backends"]


def _check(t, dtype, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("%s must be a CUDA tensor" % name)
    if t.dtype != dtype:
        raise TypeError("%s has dtype %s, expected %s" % (name, t.dtype, dtype))
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    return t.data_ptr()


class Backend:
    """GB300 backend: every operator runs as a hand-written sm_103a kernel."""

    name = "gb300"

    def __init__(self, dtype=torch.float32, stream=None):
        if dtype not in (torch.float32, torch.float64):
            raise ValueError("dtype must be float32 or float64")
        self.dtype = dtype
        self.sfx = "f32" if dtype == torch.float32 else "f64"
        self.R = F32 if dtype == torch.float32 else F64
        self.sigma_vatistas = 0.0
        self._stream = stream

    # -- helpers -----------------------------------------------------------
    def stream(self):
        s = self._stream if self._stream is not None else torch.cuda.current_stream()
        return ctypes.c_void_p(s.cuda_stream)

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

    def _vec(self, v):
        T = ctypes.c_float if self.dtype == torch.float32 else ctypes.c_double
        return (T * 3)(*[float(x) for x in v])

    def coeff_cl(self, forces, lift_axis, freestream, rho, area):
        _, nc, ns = forces.shape
        T = ctypes.c_float if self.dtype == torch.float32 else ctypes.c_double
        out = T()
        la, fs = self._vec(lift_axis), self._vec(freestream)
        call("gbvlm_coeff_cl_" + self.sfx, ns, nc, _check(forces, self.dtype, "forces"),
             ctypes.cast(la, ctypes.c_void_p), ctypes.cast(fs, ctypes.c_void_p), self.R(rho), self.R(area),
             ctypes.cast(ctypes.pointer(out), ctypes.c_void_p), self.stream())
        return out.value

    def coeff_cm(self, forces, verts_wing, ref_pt, freestream, rho, area, mac):
        _, nc, ns = forces.shape
        T = ctypes.c_float if self.dtype == torch.float32 else ctypes.c_double
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
        T = ctypes.c_float if self.dtype == torch.float32 else ctypes.c_double
        out = T()
        call("gbvlm_mesh_mac_" + self.sfx, ns, nc, _check(verts_wing, self.dtype, "verts_wing"),
             _check(areas, self.dtype, "areas"), ctypes.cast(ctypes.pointer(out), ctypes.c_void_p), self.stream())
        return out.value

    def gamma_wake_from_coeffs(self, gamma_wake, gamma_coeffs, harmonics, tn, omega, dt, iteration):
        ncols, ns = gamma_wake.shape
        call("gbvlm_gamma_wake_from_coeffs_" + self.sfx, _check(gamma_wake, self.dtype, "gamma_wake"), ns, ncols,
             _check(gamma_coeffs, self.dtype, "gamma_coeffs"), int(harmonics), self.R(tn), self.R(omega),
             self.R(dt), int(iteration), self.stream())

    def sum(self, tensor):
        T = ctypes.c_float if self.dtype == torch.float32 else ctypes.c_double
        out = T()
        call("gbvlm_sum_" + self.sfx, _check(tensor, self.dtype, "tensor"), tensor.numel(),
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
        T = ctypes.c_float if self.dtype == torch.float32 else ctypes.c_double
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

    def create_lu_solver(self):
        return LU(self)


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
        nrhs = 1 if x.dim() == 1 else x.shape[0]
        n = A.shape[0]
        call("gbvlm_lu_solve_" + b.sfx, self.h, _check(A, b.dtype, "A"), n, A.shape[1], _check(x, b.dtype, "x"),
             n, nrhs, b.stream())


def get_available_backends():
    return ["gb300"]


def create_backend(name, dtype=torch.float32):
    if name not in ("gb300", "cuda", "cpu"):
        raise RuntimeError("Unsupported backend: " + name)
    return Backend(dtype)
