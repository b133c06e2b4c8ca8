"""Coupled aeroelastic pitch-plunge simulation over the gbvlm C ABI
(``gbvlm_aero2dof_*``): the reference's UVLM_2DOF (tests/uvlm_2dof.cpp,
COUPLED branch).

``UVLM_2DOF(surfaces, lifting).run(vars, t_final)`` places the wing at a 3
degree pitch about the elastic axis, factors the AIC once, and advances the
Newton-coupled time loop on the device: float aerodynamics, double
Newmark-beta structure.  ``vars`` holds the UVLM_2DOF_Vars fields (b, k_a,
rho, a_h, omega, zeta_a, zeta_h, x_a, mu, r_a, U_a); the result holds the
nondimensional time, the plunge/pitch state u, v, a (h, alpha per row), the
generalized loads F and the Newton iterations of every step.
"""
import ctypes

import numpy as np

from ._lib import P, PP, call, dims_array
from .device import stream_handle

__all__ = ["UVLM_2DOF", "VARS_FIELDS", "reference_vars"]

VARS_FIELDS = ("b", "k_a", "rho", "a_h", "omega", "zeta_a", "zeta_h", "x_a", "mu", "r_a", "U_a")


class _Vars(ctypes.Structure):
    _fields_ = [(f, ctypes.c_double) for f in VARS_FIELDS]


def reference_vars():
    """The parameters of the reference's run (tests/uvlm_2dof.cpp:880-892)."""
    return dict(b=0.5, k_a=1000.0, rho=1.0, a_h=-0.5, omega=0.2, zeta_a=0.0, zeta_h=0.0, x_a=0.25, mu=100.0,
                r_a=0.5, U_a=7.0)


class UVLM_2DOF:
    def __init__(self, surfaces, lifting, backend="gb300"):
        """surfaces: float (4, nc+1, ns+1) vertex arrays in dimensional units
        (quarter-chord shifted); lifting: one flag per surface."""
        self.surfaces = [np.ascontiguousarray(s, np.float32) for s in surfaces]
        self.lifting = [int(x) for x in lifting]
        self.h = None

    def __del__(self):
        if getattr(self, "h", None):
            try:
                call("gbvlm_aero2dof_destroy", self.h)
            except Exception:
                pass

    def start(self, vars, t_final, stream=None):
        """Initial pose, AIC and t = 0 solve; returns (t_steps, dt)."""
        nsurf = len(self.surfaces)
        dims = dims_array([(s.shape[2] - 1, s.shape[1] - 1, 0) for s in self.surfaces])
        arr = (ctypes.c_void_p * nsurf)(*[s.ctypes.data for s in self.surfaces])
        lf = (ctypes.c_int32 * nsurf)(*self.lifting)
        vv = _Vars(**{f: float(vars[f]) for f in VARS_FIELDS})
        if self.h:
            call("gbvlm_aero2dof_destroy", self.h)
        self.h = ctypes.c_void_p()
        t_steps = ctypes.c_int64()
        dt = ctypes.c_double()
        call("gbvlm_aero2dof_create", ctypes.cast(ctypes.pointer(self.h), P), nsurf, dims, ctypes.cast(arr, PP),
             ctypes.cast(lf, P), ctypes.cast(ctypes.pointer(vv), P), float(t_final),
             ctypes.cast(ctypes.pointer(t_steps), P), ctypes.cast(ctypes.pointer(dt), P), self._s(stream))
        self.t_steps, self.dt, self.done = t_steps.value, dt.value, 0
        return self.t_steps, self.dt

    def advance(self, steps, max_iter=50, stream=None):
        """Advance `steps` coupled time steps (each a Newton loop)."""
        call("gbvlm_aero2dof_run", self.h, int(steps), int(max_iter), self._s(stream))
        self.done += int(steps)

    def results(self, stream=None):
        n = self.done
        u, v, a, F = (np.zeros((n + 1, 2)) for _ in range(4))
        iters = np.zeros(max(n, 1), np.int32)
        done = ctypes.c_int64()
        call("gbvlm_aero2dof_results", self.h, ctypes.cast(ctypes.pointer(done), P),
             *[ctypes.c_void_p(x.ctypes.data) for x in (u, v, a, F, iters)], self._s(stream))
        return dict(t=np.arange(n + 1) * self.dt, u=u, v=v, a=a, F=F, iters=iters[:n], dt=self.dt,
                    t_steps=self.t_steps)

    def run(self, vars, t_final, steps=None, max_iter=50, stream=None):
        """UVLM_2DOF::run: the whole time loop (or its first `steps` steps)."""
        t_steps, _ = self.start(vars, t_final, stream)
        n = t_steps - 2 if steps is None else min(int(steps), t_steps - 2)
        self.advance(n, max_iter, stream)
        return self.results(stream)

    @staticmethod
    def _s(stream):
        return stream_handle(stream)
