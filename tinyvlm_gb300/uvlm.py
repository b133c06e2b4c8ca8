"""Unsteady VLM driver over the gbvlm C ABI (``gbvlm_uvlm_*``).

``UVLM(backend, meshes).run(assembly, t_final)`` mirrors
vlm/src/vlm.cpp:358-509: the time step is the last panel chord of the first
surface over the body speed at t = 0, the wake grows one row per step, CL(t)
and CM_y(t) (about T_0(t) (0.5, 0, 0)) are recorded from the second step on.
The kinematics tree is evaluated on the host with dual numbers for every
step and uploaded once; the step loop runs on the device.
"""
import ctypes
import math

import numpy as np

from . import _lib
from ._lib import P, PP, call, dims_array
from .kinematics import to_colmajor
from .vlm import read_plot3d
from .device import stream_handle

__all__ = ["UVLM", "kinematics_arrays"]


def kinematics_arrays(assembly, t_steps, dt):
    """Per-step transforms, their rates, freestream and moment reference."""
    nsurf = len(assembly.surface_kinematics())
    ts = np.arange(t_steps + 1) * dt
    T = np.zeros((t_steps + 1, nsurf, 16))
    Td = np.zeros((t_steps + 1, nsurf, 16))
    for m, node in enumerate(assembly.surface_kinematics()):
        v, d = node.transform_series(ts)
        T[:, m] = v.transpose(0, 2, 1).reshape(-1, 16)
        Td[:, m] = d.transpose(0, 2, 1).reshape(-1, 16)
    _, da = assembly.kinematics().transform_series(ts)
    fs = -da[:, :3, 3]  # -(dT/dt) [0 0 0 1]: velocity of the assembly origin
    v0, _ = assembly.surface_kinematics()[0].transform_series(ts)
    ref = (v0 @ np.array([0.5, 0.0, 0.0, 1.0]))[:, :3]
    return T, Td, fs, ref


class UVLM:
    def __init__(self, backend_name, meshes, precision=32):
        if backend_name not in ("gb300", "cuda", "cpu"):
            raise RuntimeError("Unsupported backend: " + backend_name)
        self.verts = [read_plot3d(m) if isinstance(m, str) else np.ascontiguousarray(m, np.float32) for m in meshes]
        self.precision = precision
        self.h = None

    def __del__(self):
        try:
            if self.h:
                _lib.lib().gbvlm_uvlm_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def time_step(self, assembly):
        v = self.verts[0]
        d = v[:3, -1, 0].astype(np.float64) - v[:3, -2, 0].astype(np.float64)
        chord = float(np.float32(math.sqrt(float(d @ d))))
        speed = float(np.linalg.norm(assembly.kinematics().linear_velocity(0.0, (0.0, 0.0, 0.0))))
        return chord / speed

    def run(self, assembly, t_final=None, t_steps=None, dt=None, rollup=False, sigma=0.0, stream=None,
            return_gamma=False):
        dt = dt if dt is not None else self.time_step(assembly)
        if t_steps is None:
            t_steps = int(t_final / dt)
        T, Td, fs, ref = kinematics_arrays(assembly, t_steps, dt)
        from . import autotune
        npts = sum((v.shape[1] - 1) * (v.shape[2] - 1) for v in self.verts)
        # keyed by the final wake length: the last, longest wake sums take most of a run's time
        self.tuning = autotune.apply(autotune.wake_key(npts, t_steps, autotune.device_sms()))
        lifting = assembly.lifting if assembly.lifting else [True] * len(self.verts)
        dims = dims_array([(v.shape[2] - 1, v.shape[1] - 1, 0) for v in self.verts])
        arr = (ctypes.c_void_p * len(self.verts))(*[v.ctypes.data for v in self.verts])
        lf = (ctypes.c_int32 * len(self.verts))(*[1 if x else 0 for x in lifting])
        if self.h:
            _lib.lib().gbvlm_uvlm_destroy(self.h)
        h = ctypes.c_void_p()
        call("gbvlm_uvlm_create", ctypes.cast(ctypes.pointer(h), P), len(self.verts), dims, ctypes.cast(arr, PP),
             ctypes.cast(lf, P), int(t_steps), int(self.precision))
        self.h = h
        keep = [np.ascontiguousarray(x) for x in (T, Td, fs, ref)]
        call("gbvlm_uvlm_set_kinematics", h, *[ctypes.c_void_p(x.ctypes.data) for x in keep])
        s = stream_handle(stream)
        call("gbvlm_uvlm_run", h, float(dt), 1 if rollup else 0, float(sigma), s)
        cl = np.zeros(t_steps)
        cm = np.zeros((t_steps, 3))
        n = sum((v.shape[1] - 1) * (v.shape[2] - 1) for v in self.verts)
        g = np.zeros(n) if return_gamma else None
        call("gbvlm_uvlm_results", h, ctypes.c_void_p(cl.ctypes.data), ctypes.c_void_p(cm.ctypes.data),
             ctypes.c_void_p(g.ctypes.data) if g is not None else None, s)
        out = dict(t=np.arange(t_steps) * dt, cl=cl, cm=cm, dt=dt, t_steps=t_steps)
        if return_gamma:
            out["gamma"] = g
        return out
