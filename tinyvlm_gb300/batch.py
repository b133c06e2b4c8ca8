"""Batched steady solves over the gbvlm C ABI (``gbvlm_batch_*``).

Many single-surface cases of uneven size, each with several angles of attack,
solved in one CUDA graph; see include/gbvlm.h for the two formulations
(``exact``: one AIC per case and angle with the reference's alpha-dependent
geometry; ``shared``: one AIC per case, angles as right-hand sides).
"""
import collections
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
    def __init__(self, cases, mode="shared", refine=1, tuned=True, fp64_residual=False, in_flight=1):
        """``tuned``: take the plan's launch shapes from the autotuner's table
        for this workload's shape and ``in_flight``, the batches the caller
        keeps in flight at once (autotune.batch_key); otherwise the library's
        current parameters.  ``fp64_residual``: the refinement
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
                                                            autotune.device_sms(), in_flight))
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


class BatchPipeline:
    """Several batches of one workload in flight at once.

    ``depth`` solver instances (each with its own device buffers and CUDA
    graph) on their own streams, used in turn.  A batch's step ends with the
    factorisations of its largest systems, a chain of launches that leaves
    most SMs idle; with the next batch already enqueued on another stream,
    its assembly and small systems fill them.  Each batch's results are
    bitwise those of a single BatchSolver; a batch's latency grows with the
    depth, since it shares the GPU with the batches around it.

    Two ways to drive it:

    - ``submit`` / ``collect``: host inputs in, results out, first in first
      out.  ``submit`` copies the inputs and enqueues the solve on the next
      free slot, returning a ticket; ``collect`` waits for the oldest batch
      in flight and reads it back.  At most ``depth`` batches are in flight.
    - ``set_inputs`` once, then ``run``: inputs resident on the device, the
      same batch solved again on each slot in turn, nothing read back.

    ``streams``: one stream per slot (any object ``stream_handle`` accepts);
    by default the library's own non-blocking streams.
    """

    def __init__(self, cases, depth=2, mode="shared", refine=1, tuned=True, fp64_residual=False, streams=None):
        if depth < 1:
            raise ValueError("depth must be at least 1")
        if streams is None:
            from .device import Stream
            streams = [Stream() for _ in range(depth)]
        if len(streams) != depth:
            raise ValueError("need one stream per slot (%d), got %d" % (depth, len(streams)))
        self.slots = [BatchSolver(cases, mode=mode, refine=refine, tuned=tuned, fp64_residual=fp64_residual,
                                  in_flight=depth) for _ in range(depth)]
        self.streams = list(streams)
        self.depth = depth
        self.nsolve = self.slots[0].nsolve
        self.gamma_floats = self.slots[0].gamma_floats
        self.tuning = self.slots[0].tuning
        self._turn = 0  # the slot the next batch goes to
        self._inflight = collections.deque()  # (ticket, slot, want_gamma), oldest first
        self._tickets = 0

    def pending(self):
        """Batches submitted and not yet collected."""
        return len(self._inflight)

    def full(self):
        return len(self._inflight) == self.depth

    def submit(self, verts, alphas, u_inf=1.0, rho=1.0, ref_pt=(0.0, 0.0, 0.0), want_gamma=False):
        """Copy one batch's inputs to the next free slot and enqueue its solve;
        returns the batch's ticket.  The inputs are as for
        BatchSolver.set_inputs; the call returns once they are copied."""
        if self.full():
            raise RuntimeError("all %d slots hold a batch: collect one first" % self.depth)
        # first in first out over a ring: the slots in flight are the `pending`
        # ones before _turn, so _turn itself is free
        slot = self._turn
        s, st = self.slots[slot], self.streams[slot]
        s.set_inputs(verts, alphas, u_inf=u_inf, rho=rho, ref_pt=ref_pt, stream=st)
        s.run(want_gamma=want_gamma, stream=st)
        self._turn = (slot + 1) % self.depth
        ticket = self._tickets
        self._tickets += 1
        self._inflight.append((ticket, slot, bool(want_gamma)))
        return ticket

    def collect(self, co=None, g=None):
        """Wait for the oldest batch in flight and read it back: coefficients
        (nsolve, 5) into ``co`` (allocated when None), circulations into
        ``g`` when that batch was submitted with want_gamma.  Returns
        (ticket, co, g).  Status errors of the batch raise as in
        BatchSolver.results."""
        if not self._inflight:
            raise RuntimeError("no batch in flight")
        ticket, slot, wg = self._inflight[0]
        if g is not None and not wg:
            raise ValueError("batch %d was submitted without want_gamma" % ticket)
        if co is None:
            co = np.zeros((self.nsolve, 5), np.float64)
        self._inflight.popleft()
        self.slots[slot].results_into(co, g, stream=self.streams[slot])
        return ticket, co, g

    def set_inputs(self, verts, alphas, u_inf=1.0, rho=1.0, ref_pt=(0.0, 0.0, 0.0)):
        """The same inputs on every slot, for ``run``."""
        if self._inflight:
            raise RuntimeError("collect the batches in flight first")
        for s, st in zip(self.slots, self.streams):
            s.set_inputs(verts, alphas, u_inf=u_inf, rho=rho, ref_pt=ref_pt, stream=st)

    def run(self, want_gamma=False):
        """Enqueue one solve of the resident inputs on the next slot's stream;
        returns the slot.  Nothing is read back."""
        if self._inflight:
            raise RuntimeError("collect the batches in flight first")
        slot = self._turn
        self.slots[slot].run(want_gamma=want_gamma, stream=self.streams[slot])
        self._turn = (slot + 1) % self.depth
        return slot

    def launches(self):
        """Kernel launches of one batch."""
        return self.slots[0].launches()


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
