"""Structural time integration on the device: class NewmarkBeta of the
reference (vlm/include/vlm_integrator.hpp:7-41) over the C ABI
(gbvlm_newmark_*), in double.

Matrices and vectors are float64 device arrays (``device.DeviceArray`` or any
object with ``data_ptr()`` and ``shape``).  Matrices are read column-major,
element (r, c) at r + c * ndof, like the reference's TensorView2fD: upload
the transpose of a row-major matrix (or the matrix itself, for the symmetric
mass, damping and stiffness matrices).
"""
import ctypes

from ._lib import P, call
from .device import stream_handle as _s


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


class NewmarkBeta:
    """Newmark-beta, incremental form (vlm/src/vlm_integrator.cpp:5-68)."""

    def __init__(self, backend=None, beta=0.25, gamma=0.5):
        self.h = ctypes.c_void_p()
        call("gbvlm_newmark_create", ctypes.cast(ctypes.pointer(self.h), P), float(beta), float(gamma))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            try:
                call("gbvlm_newmark_destroy", h)
            except Exception:
                pass

    def init(self, M, C, K, dt, stream=None):
        """K_eff = K + M/(beta dt^2) + gamma C/(beta dt), factored on the device."""
        n = int(M.shape[0])
        for X in (M, C, K):
            if len(X.shape) != 2 or tuple(X.shape) != (n, n) or (hasattr(X, "is_contiguous") and not X.is_contiguous()):
                raise ValueError("Newmark matrices must be contiguous (ndof, ndof) device arrays")
        call("gbvlm_newmark_init", self.h, n, _p(M), _p(C), _p(K), float(dt), _s(stream))

    def step(self, M, C, v_i, a_i, du, dv, da, delta_F, dt, stream=None):
        """du, dv, da (written in place) of one step from v_i, a_i and delta_F."""
        call("gbvlm_newmark_step", self.h, _p(M), _p(C), _p(v_i), _p(a_i), _p(du), _p(dv), _p(da), _p(delta_F),
             float(dt), _s(stream))
