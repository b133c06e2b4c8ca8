"""Batched steady solves over the gbvlm C ABI (``gbvlm_batch_*``).

Many single-surface cases of uneven size, each with several angles of attack,
solved in one CUDA graph; see include/gbvlm.h for the two formulations
(``exact``: one AIC per case and angle with the reference's alpha-dependent
geometry; ``shared``: one AIC per case, angles as right-hand sides).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import P, call, dims_array
from .device import stream_handle

MODES = {"exact": 0, "shared": 1}
FP64_RESIDUAL = 1  # GBVLM_BATCH_FP64_RESIDUAL
STAGES = ("geometry", "assembly", "rhs", "lu_factor", "solve_refine", "loads")


def pack_verts(cases):
    """Concatenate every case's (4, nc+1, ns+1) float32 vertices."""
    return np.ascontiguousarray(np.concatenate([np.ascontiguousarray(c.verts, np.float32).ravel() for c in cases]))


def pack_alphas(cases):
    return np.ascontiguousarray(np.concatenate([np.asarray(c.alphas, np.float64) for c in cases]))


class BatchSolver:
    def __init__(self, cases, mode="shared", refine=1, tuned=True, fp64_residual=False):
        """``tuned``: take the plan's launch shapes from the autotuner's table
        for this workload's shape (autotune.batch_key); otherwise the
        library's current parameters.  ``fp64_residual``: the refinement
        residual measures the FP64 system (GBVLM_BATCH_FP64_RESIDUAL: a
        float-pair evaluation of the AIC corrects the stored float one), so
        the circulations, not only CL/CM, converge to the FP64 solution;
        needs refine >= 1."""
        self.mode = mode
        self.fp64_residual = bool(fp64_residual)
        self.tuning = None
        if tuned:
            from . import autotune
            self.tuning = autotune.apply(autotune.batch_key([(c.ns, c.nc) for c in cases],
                                                            [len(c.alphas) for c in cases], mode, refine,
                                                            autotune.device_sms()))
        self.dims = [(c.ns, c.nc, 0) for c in cases]
        self.nalpha = [len(c.alphas) for c in cases]
        d = dims_array(self.dims)
        na = (ctypes.c_int32 * len(cases))(*self.nalpha)
        h = ctypes.c_void_p()
        call("gbvlm_batch_create_ex", ctypes.cast(ctypes.pointer(h), P), len(cases), d, ctypes.cast(na, P),
             MODES[mode], int(refine), FP64_RESIDUAL if fp64_residual else 0)
        self.h = h
        ns, nsys, gf = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        inter, luf, ab = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        call("gbvlm_batch_info", h, *[ctypes.cast(ctypes.pointer(x), P) for x in (ns, nsys, gf, inter, luf, ab)])
        self.nsolve, self.nsys, self.gamma_floats = ns.value, nsys.value, gf.value
        self.interactions, self.lu_flops, self.arena_bytes = inter.value, luf.value, ab.value
        self.n_per_solve = [c.ns * c.nc for c in cases for _ in c.alphas]

    def __del__(self):
        try:
            if self.h:
                _lib.lib().gbvlm_batch_destroy(self.h)
                self.h = None
        except Exception:
            pass

    @staticmethod
    def _ptr(x):
        if hasattr(x, "data_ptr"):
            return ctypes.c_void_p(x.data_ptr())
        return ctypes.c_void_p(x.ctypes.data)

    def set_inputs(self, verts, alphas, u_inf=1.0, rho=1.0, ref_pt=(0.0, 0.0, 0.0), stream=None):
        """verts: packed float32 vertices (numpy, pinned torch CPU tensor or CUDA tensor); alphas: host float64."""
        self._alphas = np.ascontiguousarray(alphas, np.float64)
        rp = (ctypes.c_double * 3)(*ref_pt)
        call("gbvlm_batch_set_inputs", self.h, self._ptr(verts), ctypes.c_void_p(self._alphas.ctypes.data),
             float(u_inf), float(rho), ctypes.cast(rp, P), self._s(stream))

    @staticmethod
    def _s(stream):
        return stream_handle(stream)

    def run(self, want_gamma=False, stream=None, graph=True):
        """Enqueue the solve; graph=False launches it kernel by kernel (a batch solved once)."""
        call("gbvlm_batch_run" if graph else "gbvlm_batch_run_eager", self.h, 1 if want_gamma else 0,
             self._s(stream))

    def results(self, gamma=False, stream=None):
        co = np.zeros((self.nsolve, 5), np.float64)
        g = np.zeros(self.gamma_floats, np.float32) if gamma else None
        call("gbvlm_batch_results", self.h, ctypes.c_void_p(co.ctypes.data),
             ctypes.c_void_p(g.ctypes.data) if g is not None else None, self._s(stream))
        if not gamma:
            return co, None
        out, off = [], 0
        for n in self.n_per_solve:
            out.append(g[off:off + n])
            off += n
        return co, out

    def results_into(self, co, g=None, stream=None):
        """Read back into caller-owned (pinned) host arrays; returns bytes copied."""
        call("gbvlm_batch_results", self.h, ctypes.c_void_p(co.ctypes.data),
             ctypes.c_void_p(g.ctypes.data) if g is not None else None, self._s(stream))
        return co.nbytes + (g.nbytes if g is not None else 0)

    def launches(self):
        v = ctypes.c_int64()
        call("gbvlm_batch_launches", self.h, ctypes.cast(ctypes.pointer(v), P))
        return v.value

    def profile(self, stream=None):
        """Run the stages eagerly, each bracketed by CUDA events on `stream`;
        returns milliseconds per stage (STAGES order)."""
        ms = (ctypes.c_float * len(STAGES))()
        call("gbvlm_batch_profile", self.h, ctypes.cast(ms, P), self._s(stream))
        return dict(zip(STAGES, list(ms)))

    def update_profile(self, stream=None):
        """CUDA-event time of the LU's tensor-core trailing-update launches in
        one eager run, with their algorithmic flops and bytes."""
        out = (ctypes.c_double * 4)()
        call("gbvlm_batch_update_profile", self.h, ctypes.cast(out, P), self._s(stream))
        return {"ms": out[0], "launches": int(out[1]), "flops": out[2], "bytes": out[3]}


def smoke_check():
    """Tiny batch through the C ABI checked against the oracle (used by smoke())."""
    from oracle import oracle as O
    from . import mesh as M
    cases = M.batch_cases(3, seed=7, n_alpha=2, nc_range=(4, 6), ns_range=(4, 8))
    for mode in ("shared", "exact"):
        bs = BatchSolver(cases, mode=mode, refine=1)
        bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=(0.25, 0.0, 0.0))
        bs.run()
        co, _ = bs.results()
        k = 0
        for c in cases:
            v64 = c.verts.astype(np.float64)
            refs = (O.vlm_shared([v64], c.alphas, ref_pt=(0.25, 0, 0)) if mode == "shared"
                    else [O.vlm_run([v64], a, dtype=np.float64, ref_pt=(0.25, 0, 0)) for a in c.alphas])
            for r in refs:
                cl = float(r["cl"])
                assert abs(co[k, 0] - cl) <= 1e-5 * max(abs(cl), 1e-3), ("batch smoke", mode, co[k, 0], cl)
                k += 1
