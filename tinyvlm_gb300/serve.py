"""Served mixed stream: continuous batching of steady VLM solves, UVLM
single-step advances of a resident unsteady case, and harmonic-balance
(HBVLM) residual evaluations on one GPU.

Design
------
* ``lanes`` dispatcher threads, each with its own CUDA stream (a slot on the
  device); the library calls release the GIL, so the work of different
  lanes overlaps on the device.
* One FIFO queue.  A lane that takes a steady request also takes every
  other steady request already waiting (continuous batching) up to
  ``max_batch`` cases and the free HBM budget, and solves them as one
  batched plan (``tinyvlm_gb300.batch``, one refinement sweep); requests
  arriving meanwhile wait for the next free lane.
* Admission by HBM budget: the budget is the smaller of ``hbm_budget`` and
  the device memory free when the server starts; each request reserves its
  device footprint (AIC and work arrays of its batch) before launch and
  releases it when done; a request that does not fit waits at the head of
  the queue.
* Every wait is bounded: lanes sleep on the queue's condition until a
  request or shutdown arrives, and a reservation, a UVLM step's turn or a
  request's completion that takes longer than ``wait_s`` fails with
  TimeoutError instead of hanging the server.
* The UVLM case (wing, wake, AIC factors) and one HBVLM engine per lane
  stay resident on the device; a UVLM request advances the case by one time
  step (steps run in arrival order, they depend on each other), an HBVLM
  request runs the harmonic-balance fixed point for its own frequency and
  amplitudes from rest.
* UVLM requests bypass the lanes: they go to a device-resident request loop
  (``device_loop``, gbvlm_uvlm_loop_*).  Submitting one raises a counter in
  mapped host memory; a CUDA graph running on the GPU takes the step, writes
  its coefficients back and waits (on the GPU, bounded by ``poll_s``) for
  the next request, so back-to-back steps make no CUDA call at all.  One
  host thread collects the completions in ticket order.

Every result carries its arrival, start and finish times; ``latency`` is
finish - arrival.
"""
import collections
import math
import threading
import time

import numpy as np

from . import mesh as M
from .batch import BatchSolver, pack_alphas, pack_verts
from .device import Stream, stream_handle


class Request:
    __slots__ = ("rid", "kind", "payload", "arrival", "start", "finish", "result", "error", "done")

    def __init__(self, rid, kind, payload, arrival=None):
        self.rid, self.kind, self.payload = rid, kind, payload
        self.arrival = time.perf_counter() if arrival is None else arrival
        self.start = self.finish = None
        self.result = self.error = None
        self.done = threading.Event()

    @property
    def latency(self):
        return None if self.finish is None else self.finish - self.arrival


def steady_bytes(n, nalpha=1):
    """Device footprint of one steady system in the batched engine (AIC plus per-panel and per-solve arrays)."""
    return 4 * n * n + 200 * n + 64 * n * nalpha + 4096


class Server:
    def __init__(self, lanes=3, hbm_budget=32 << 30, max_batch=64, uvlm=None, hbvlm=None, mode="exact", refine=1,
                 wait_s=120.0, device_loop=True, poll_s=0.05):
        from .device import device_info
        self.lanes = lanes
        free = device_info()[1]
        self.budget = int(min(hbm_budget, free))
        self.refine = refine
        self.wait_s = float(wait_s)
        self.used = 0
        self.max_batch = max_batch
        self.mode = mode
        self.q = collections.deque()
        self.cv = threading.Condition()
        self.stop = False
        self.uvlm = uvlm          # resident unsteady case, or None
        self.uvlm_cv = threading.Condition()
        self.uvlm_next_ticket = 0  # issued at dequeue time: steps run in arrival order
        self.uvlm_turn = 0
        self.hbvlm_factory = hbvlm
        self.device_loop = device_loop and uvlm is not None
        self.poll_s = poll_s
        self.uloop = None
        self.device_loop_error = None
        self.uq = collections.deque()
        self.ucv = threading.Condition()
        self.threads = []
        self.stats = collections.Counter()

    # -- resident state -----------------------------------------------------
    def reserve(self, nbytes, block=True):
        """Reserve device bytes of the budget; waits (bounded) for releases."""
        deadline = time.monotonic() + self.wait_s
        with self.cv:
            while self.used + nbytes > self.budget:
                left = deadline - time.monotonic()
                if not block:
                    return False
                if left <= 0:
                    raise TimeoutError("no %d bytes of the device budget freed within %.0f s" % (nbytes, self.wait_s))
                self.cv.wait(left)
            self.used += nbytes
            return True

    def release(self, nbytes):
        with self.cv:
            self.used -= nbytes
            self.cv.notify_all()

    # -- lifecycle ----------------------------------------------------------
    def start(self):
        for k in range(self.lanes):
            t = threading.Thread(target=self._lane, args=(k,), daemon=True)
            t.start()
            self.threads.append(t)
        if self.device_loop:
            from ._lib import GbvlmError
            try:
                self.uloop = UvlmLoop(self.uvlm, self.poll_s)
            except GbvlmError as e:  # e.g. no native atomics on host memory: the lanes step the case
                self.device_loop = False
                self.stats["device_loop_unavailable"] += 1
                self.device_loop_error = str(e)
        if self.device_loop:
            t = threading.Thread(target=self._uvlm_completions, daemon=True)
            t.start()
            self.threads.append(t)
        return self

    def shutdown(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        with self.ucv:
            self.ucv.notify_all()
        for t in self.threads:
            t.join()
        if self.uloop is not None:
            self.uloop.close()
            self.uloop = None

    def submit(self, req):
        if req.kind == "uvlm" and self.uloop is not None:
            with self.ucv:  # tickets and the completion queue in the same order
                req.start = time.perf_counter()
                req.payload = self.uloop.submit()
                self.uq.append(req)
                self.ucv.notify()
            return req
        with self.cv:
            self.q.append(req)
            self.cv.notify()
        return req

    def _uvlm_completions(self):
        """Completions of the device loop, in ticket order."""
        while True:
            with self.ucv:
                while not self.uq and not self.stop:
                    self.ucv.wait()
                if not self.uq:
                    return
                req = self.uq.popleft()
            try:
                req.result = self.uloop.wait(req.payload, self.wait_s)
            except Exception as e:  # the request fails, the loop keeps serving
                req.error = e
            req.finish = time.perf_counter()
            req.done.set()
            self.stats["uvlm_loop_steps"] += 1

    # -- workers ------------------------------------------------------------
    def _take(self):
        with self.cv:
            while not self.q and not self.stop:
                self.cv.wait()  # submit() and shutdown() notify
            if not self.q:
                return None
            head = self.q.popleft()
            group = [head]
            if head.kind == "uvlm":
                head.payload = self.uvlm_next_ticket
                self.uvlm_next_ticket += 1
            if head.kind == "steady":
                need = steady_bytes(head.payload[0].n, len(head.payload[0].alphas))
                keep = collections.deque()
                while self.q and len(group) < self.max_batch:
                    r = self.q.popleft()
                    if r.kind == "steady":
                        b = steady_bytes(r.payload[0].n, len(r.payload[0].alphas))
                        if self.used + need + b <= self.budget:
                            group.append(r)
                            need += b
                            continue
                    keep.append(r)
                self.q.extendleft(reversed(keep))
            return group

    def _lane(self, k):
        stream = Stream()
        hb = self.hbvlm_factory() if self.hbvlm_factory else None
        while True:
            group = self._take()
            if group is None:
                return
            t0 = time.perf_counter()
            for r in group:
                r.start = t0
            try:
                kind = group[0].kind
                if kind == "steady":
                    self._steady(group, stream)
                elif kind == "uvlm":
                    self._uvlm(group[0], stream)
                elif kind == "hbvlm":
                    self._hbvlm(group[0], hb)
                else:
                    raise ValueError("unknown request kind " + kind)
            except Exception as e:  # the request fails, the lane keeps serving
                for r in group:
                    r.error = e
            t1 = time.perf_counter()
            for r in group:
                r.finish = t1
                r.done.set()
            self.stats[group[0].kind + "_groups"] += 1

    def _steady(self, group, stream):
        cases = [r.payload[0] for r in group]
        need = sum(steady_bytes(c.n, len(c.alphas)) for c in cases)
        if need > self.budget:
            raise MemoryError("steady request needs %d bytes, above the %d-byte device budget" % (need, self.budget))
        self.reserve(need)
        try:
            bs = BatchSolver(cases, mode=self.mode, refine=self.refine)
            bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=(0.25, 0.0, 0.0), stream=stream)
            bs.run(want_gamma=False, stream=stream, graph=False)  # solved once: no graph capture
            co, _ = bs.results(stream=stream)
            del bs
        finally:
            self.release(need)
        k = 0
        for r, c in zip(group, cases):
            r.result = co[k:k + len(c.alphas)].copy()
            k += len(c.alphas)
        self.stats["steady_solves"] += k

    def _uvlm(self, req, stream):
        import ctypes
        from ._lib import P, call
        ticket = req.payload
        deadline = time.monotonic() + self.wait_s
        with self.uvlm_cv:
            while self.uvlm_turn != ticket:
                left = deadline - time.monotonic()
                if left <= 0:
                    raise TimeoutError("UVLM step %d did not get its turn within %.0f s" % (ticket, self.wait_s))
                self.uvlm_cv.wait(left)
        try:
            sim = self.uvlm
            step = ctypes.c_int64()
            cl = ctypes.c_double()
            cm = (ctypes.c_double * 3)()
            call("gbvlm_uvlm_step", sim.h, ctypes.cast(ctypes.pointer(step), P), ctypes.cast(ctypes.pointer(cl), P),
                 ctypes.cast(cm, P), stream_handle(stream))
            req.result = (step.value, cl.value, tuple(cm))
        finally:
            with self.uvlm_cv:
                self.uvlm_turn += 1
                self.uvlm_cv.notify_all()

    def _hbvlm(self, req, hb):
        omega, dyn = req.payload
        ft = np.zeros((2, dyn.shape[1]))
        hb.gamma_coeffs[:] = 0.0  # each residual evaluation starts from rest, independent of order
        hb.run(omega, dyn, ft)
        req.result = ft


# ---------------------------------------------------------------------------
# workload helpers
# ---------------------------------------------------------------------------
def steady_case(rng, n_lo=256, n_hi=16384):
    """Random trapezoid with a panel count log-uniform in [n_lo, n_hi]."""
    n = int(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi))))
    nc = int(np.clip(round(math.sqrt(n / 4.0)), 4, 64))
    ns = int(np.clip(round(n / nc), 4, 512))
    ar = float(rng.uniform(4, 12))
    lam = float(rng.uniform(0.3, 1.0))
    sw = float(rng.uniform(0, 35))
    v = M.trapezoid(nc, ns, ar, lam, sw).astype(np.float32)
    M.quarter_chord(v)
    return M.Case(v, np.radians([rng.uniform(-8, 8)]), dict(nc=nc, ns=ns))


def resident_uvlm(ns=80, nc=20, warm_steps=500, capacity=4096, rollup=False):
    """The resident unsteady case: 20 x 80 pitch-plunge wing advanced
    ``warm_steps`` steps (wake of warm_steps x ns rings); ``capacity`` bounds
    the further steps it can serve.  The warm-up steps run on the legacy
    default stream; the served steps run on the lanes' non-blocking streams,
    which do not order themselves after it, so the warm-up ends with a device
    synchronisation."""
    import ctypes
    from . import _lib
    from ._lib import P, PP, call, dims_array
    from .kinematics import Assembly, KinematicsTree, rotation_matrix, sin, translation_matrix
    from .uvlm import kinematics_arrays
    v = M.rectangular(nc, ns, 1.0, 4.0).astype(np.float32)
    M.quarter_chord(v)
    k = 0.5
    tree = KinematicsTree()
    fs = tree.add(lambda t: translation_matrix([-t, 0.0, 0.0]))
    heave = tree.add(lambda t: translation_matrix([0.0, 0.0, 0.1 * sin(k * t)])).after(fs)
    pitch = tree.add(lambda t: rotation_matrix([0.25, 0, 0], [0, 1, 0], math.radians(3.0) * sin(k * t + math.pi / 2))).after(heave)
    asm = Assembly(fs)
    asm.add("wing", pitch)
    t_steps = warm_steps + capacity + 2
    T, Td, fsv, ref = kinematics_arrays(asm, t_steps, 0.05)

    class Sim:
        pass

    sim = Sim()
    sim.verts = v
    sim.assembly = asm
    d = dims_array([(ns, nc, 0)])
    arr = (ctypes.c_void_p * 1)(v.ctypes.data)
    lf = (ctypes.c_int32 * 1)(1)
    h = ctypes.c_void_p()
    call("gbvlm_uvlm_create", ctypes.cast(ctypes.pointer(h), P), 1, d, ctypes.cast(arr, PP), ctypes.cast(lf, P),
         int(t_steps), 32)
    sim.h = h
    sim.keep = [np.ascontiguousarray(x) for x in (T, Td, fsv, ref)]
    call("gbvlm_uvlm_set_kinematics", h, *[ctypes.c_void_p(x.ctypes.data) for x in sim.keep])
    call("gbvlm_uvlm_begin", h, 0.05, 1 if rollup else 0, 0.0, None)
    for _ in range(warm_steps):
        call("gbvlm_uvlm_step", h, None, None, None, None)
    call("gbvlm_device_synchronize")
    return sim


class UvlmLoop:
    """The device-resident request loop of a resident UVLM case
    (gbvlm_uvlm_loop_*): submit() returns a ticket at once, wait() returns
    that step's (step index, CL, CM) when the GPU has taken it."""

    def __init__(self, sim, poll_s=0.05):
        import ctypes
        from ._lib import P, call
        self.h = ctypes.c_void_p()
        call("gbvlm_uvlm_loop_create", ctypes.cast(ctypes.pointer(self.h), P), sim.h, float(poll_s))

    def submit(self):
        import ctypes
        from ._lib import P, call
        t = ctypes.c_int64()
        call("gbvlm_uvlm_loop_submit", self.h, ctypes.cast(ctypes.pointer(t), P))
        return t.value

    def wait(self, ticket, timeout_s=120.0):
        import ctypes
        from ._lib import P, call
        step, cl, cm = ctypes.c_int64(), ctypes.c_double(), (ctypes.c_double * 3)()
        call("gbvlm_uvlm_loop_wait", self.h, int(ticket), float(timeout_s), ctypes.cast(ctypes.pointer(step), P),
             ctypes.cast(ctypes.pointer(cl), P), ctypes.cast(cm, P))
        return step.value, cl.value, tuple(cm)

    def stats(self):
        import ctypes
        from ._lib import P, call
        v = [ctypes.c_int64() for _ in range(3)]
        call("gbvlm_uvlm_loop_stats", self.h, *[ctypes.cast(ctypes.pointer(x), P) for x in v])
        return {"submitted": v[0].value, "completed": v[1].value, "launches": v[2].value}

    def close(self):
        from ._lib import call
        if self.h:
            call("gbvlm_uvlm_loop_destroy", self.h)
            self.h = None


def hbvlm_factory(nc=45, harmonics=5):
    """2-DOF pitch-heave section wing (nc chordwise x 1 spanwise)."""
    from .hbvlm import HBVLM2

    def make():
        v = M.rectangular(nc, 1, 1.0, 40000.0)
        hb = HBVLM2("gb300", v)
        hb.init(harmonics, 1.0)
        return hb

    return make


def hbvlm_request(rng, harmonics=5):
    omega = float(rng.uniform(0.2, 0.6))
    dyn = np.zeros((2, 2 * harmonics + 1))
    dyn[0, 1:3] = rng.uniform(-0.02, 0.02, 2)
    dyn[1, 0] = rng.uniform(-0.02, 0.02)
    dyn[1, 1:3] = rng.uniform(-0.04, 0.04, 2)
    return omega, dyn
