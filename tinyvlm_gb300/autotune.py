"""Launch-shape autotuner.

The kernels' launch shapes are named integer parameters of the library
(gbvlm_tune_*, include/gbvlm.h): the batch LU's size-group boundaries, the
batch loads block, the batch assembly's span chunk and ring rows per tile, the split-K slice count
of the wake sums and of the HBVLM wake operator.  The reference fixes its
shapes (kernel_influence at (32, 16) blocks, vlm_backend_cuda.cu:171); here
they are searched per workload shape and kept in a table.

* ``*_key(...)`` names a workload's shape: its kind, the device's SM count
  and its sizes rounded to powers of two, so that nearby workloads share an
  entry.  A key depends only on the sizes, never on their order.
* ``lookup(key)`` returns the table's parameters for a key, or None.  The
  table is ``tuning/gb300.json`` beside this file, committed with the
  package; it is read once.
* ``apply(key)`` sets the library's parameters to the table's entry (or the
  defaults) and says which it used; the solvers call it before they build a
  plan or launch, so a tuned shape is used without the caller's help.
* ``tune_batch`` / ``tune_wake`` search on the device by coordinate descent
  (each parameter in turn over its candidates, the others held), timing
  with CUDA events, and ``save`` writes the winners into the table.

Run ``python -m tinyvlm_gb300.autotune`` on a GPU to tune the benchmark's
workloads and rewrite the table.
"""
import ctypes
import json
import math
import os
import time

import numpy as np

from . import _lib
from ._lib import P, call

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning", "gb300.json")

_TABLE = None


# ---------------------------------------------------------------------------
# the library's parameters
# ---------------------------------------------------------------------------
def params():
    """{name: (lo, hi)} of every tuning parameter the library has."""
    n = ctypes.c_int32()
    call("gbvlm_tune_count", ctypes.cast(ctypes.pointer(n), P))
    out = {}
    for i in range(n.value):
        name, lo, hi = ctypes.c_char_p(), ctypes.c_int64(), ctypes.c_int64()
        call("gbvlm_tune_name", i, ctypes.cast(ctypes.pointer(name), P), ctypes.cast(ctypes.pointer(lo), P),
             ctypes.cast(ctypes.pointer(hi), P))
        out[name.value.decode()] = (lo.value, hi.value)
    return out


def get(name):
    v = ctypes.c_int64()
    call("gbvlm_tune_get", name.encode(), ctypes.cast(ctypes.pointer(v), P))
    return v.value


def set_params(values):
    for name, v in values.items():
        call("gbvlm_tune_set", name.encode(), int(v))


def reset():
    call("gbvlm_tune_reset")


def current():
    return {name: get(name) for name in params()}


def defaults():
    saved = current()
    reset()
    d = current()
    set_params(saved)
    return d


# ---------------------------------------------------------------------------
# shape keys and the table
# ---------------------------------------------------------------------------
def _p2(x):
    """x rounded to the nearest power of two (at least 1)."""
    return 1 << max(0, int(round(math.log2(max(1, int(x))))))


def batch_key(ns_nc, nalpha, mode, refine, sms, in_flight=1):
    """A batched steady workload: cases (ns, nc), angles per case, formulation,
    refinement sweeps, the device's SM count and, when more than one, the
    batches in flight at once (BatchPipeline: other batches take the SMs a
    batch leaves idle, which moves the best size groups)."""
    n = [int(a) * int(b) for a, b in ns_nc]
    key = "batch/%s/r%d/sm%d/c%d/p%d/m%d/a%d" % (mode, int(refine), int(sms), _p2(len(n)), _p2(sum(n)), _p2(max(n)),
                                                int(max(nalpha)))
    return key + ("/f%d" % int(in_flight) if int(in_flight) > 1 else "")


def wake_key(points, rows, sms):
    """The wake sums: collocation points and active wake ring rows (all surfaces)."""
    return "wake/sm%d/p%d/r%d" % (int(sms), _p2(points), _p2(rows))


def hbvlm_key(n, instances, rows, sms):
    """The HBVLM wake operator: panels, time instances (all sets) and wake rows per instance."""
    return "hbvlm/sm%d/n%d/i%d/r%d" % (int(sms), _p2(n), _p2(instances), _p2(rows))


def table():
    global _TABLE
    if _TABLE is None:
        if os.path.exists(TABLE):
            with open(TABLE) as f:
                _TABLE = json.load(f)
        else:
            _TABLE = {"version": 1, "entries": {}}
    return _TABLE


def lookup(key):
    """The table's parameters for ``key``, or None."""
    e = table()["entries"].get(key)
    return dict(e["params"]) if e else None


def apply(key, fallback=None):
    """Set the library's parameters of ``key``'s kind from the table (or the
    defaults, or ``fallback``); returns {"key", "params", "source"}."""
    kind = key.split("/", 1)[0]
    mine = {k: v for k, v in defaults().items() if k.startswith(kind + ".")}
    found = lookup(key)
    src = "table" if found else ("given" if fallback else "default")
    mine.update(found or fallback or {})
    set_params(mine)
    return {"key": key, "params": mine, "source": src}


def save(key, best, extra=None):
    t = table()
    e = {"params": dict(best)}
    e.update(extra or {})
    t["entries"][key] = e
    os.makedirs(os.path.dirname(TABLE), exist_ok=True)
    with open(TABLE, "w") as f:
        json.dump(t, f, indent=1, sort_keys=True)


def device_sms():
    from .device import device_info
    return device_info()[0]


# ---------------------------------------------------------------------------
# searches (GPU)
# ---------------------------------------------------------------------------
def _descend(space, run, base, repeats=3):
    """Coordinate descent: each group of parameters in turn over its
    candidates, the others at their best so far; the time of a point is the
    median of `repeats` measurements."""
    best = dict(base)
    tried = []

    def measure(p):
        ts = sorted(run(p) for _ in range(repeats))
        return ts[len(ts) // 2]

    best_ms = measure(best)
    base_ms = best_ms
    tried.append({"params": dict(best), "ms": best_ms})
    for cands in space:
        for c in cands:
            p = dict(best)
            p.update(c)
            if p == best:
                continue
            try:
                ms = measure(p)
            except _lib.GbvlmError as e:  # an invalid combination is skipped
                tried.append({"params": p, "error": str(e)})
                continue
            tried.append({"params": p, "ms": ms})
            if ms < best_ms:
                best, best_ms = p, ms
    return best, best_ms, base_ms, tried


BATCH_SPACE = [
    [{"batch.group_hi": hi, "batch.group_mid": mid, "batch.group_lo": lo} for hi, mid, lo in
     ((1024, 0, 384), (1536, 0, 512), (768, 0, 320), (1024, 0, 256), (1280, 0, 448), (896, 0, 384), (2048, 0, 512),
      (1024, 0, 512), (1280, 0, 640), (2048, 0, 768), (768, 0, 256), (640, 0, 256), (896, 0, 320), (768, 0, 384),
      (1280, 768, 384), (1024, 640, 320), (1536, 896, 448), (1280, 640, 320), (1024, 512, 256), (768, 512, 256))],
    [{"batch.assembly_span": s} for s in (64, 128, 256)],
    [{"batch.assembly_rows": r} for r in (1, 2, 3, 4)],
    [{"batch.loads_threads": t} for t in (0, 32, 64, 128, 256)],
]


def tune_batch(cases, mode="shared", refine=1, steps=5, repeats=3, persist=True, in_flight=1):
    """Search the batch plan's shapes for these cases on the device; the time
    of a point is a CUDA-event measurement of `steps` graph replays per slot,
    with `in_flight` batches in flight (BatchPipeline, one stream per slot,
    every slot's last batch finished before the closing event)."""
    from .batch import BatchPipeline, pack_alphas, pack_verts
    from .device import DeviceArray, Event, Stream
    sms = device_sms()
    key = batch_key([(c.ns, c.nc) for c in cases], [len(c.alphas) for c in cases], mode, refine, sms, in_flight)
    verts = DeviceArray.from_numpy(pack_verts(cases))
    alphas = pack_alphas(cases)

    def run(p):
        set_params(p)
        pipe = BatchPipeline(cases, depth=in_flight, mode=mode, refine=refine, tuned=False)
        pipe.set_inputs(verts, alphas, ref_pt=(0.25, 0.0, 0.0))
        for _ in range(2 * in_flight):
            pipe.run()
        for st in pipe.streams:
            st.synchronize()
        # the slots' streams are independent: time each slot's replays with its
        # own events, all slots enqueued together; a point's time per batch is
        # the span from the earliest start to the latest end over all batches
        e0 = [Event() for _ in pipe.streams]
        e1 = [Event() for _ in pipe.streams]
        for e, st in zip(e0, pipe.streams):
            e.record(st)
        for _ in range(steps * in_flight):
            pipe.run()
        for e, st in zip(e1, pipe.streams):
            e.record(st)
        for st in pipe.streams:
            st.synchronize()
        first = min(range(in_flight), key=lambda i: e0[0].elapsed_time(e0[i]))
        span = max(e0[first].elapsed_time(e1[i]) for i in range(in_flight))
        del pipe
        return span / (steps * in_flight)

    base = {k: v for k, v in defaults().items() if k.startswith("batch.")}
    t0 = time.perf_counter()
    best, best_ms, base_ms, tried = _descend(BATCH_SPACE, run, base, repeats)
    out = {"key": key, "params": best, "ms": best_ms, "default_ms": base_ms, "points": len(tried),
           "search_s": time.perf_counter() - t0}
    if persist:
        save(key, best, {"ms": best_ms, "default_ms": base_ms, "tried": tried})
    reset()
    return out


WAKE_SPACE = [[{"wake.waves": w} for w in (1, 2, 4, 8, 16)]]


def tune_wake(points_ns_nc, rows, steps=5, repeats=3, persist=True):
    """Search the split-K slice count of the float wake sums for one wing of
    (ns, nc) panels with `rows` active wake ring rows."""
    from .backend import Backend
    from .device import DeviceArray, Event, Stream
    from . import mesh as M
    ns, nc = points_ns_nc
    sms = device_sms()
    key = wake_key(ns * nc, rows, sms)
    v = M.rectangular(nc, ns, 1.0, 4.0).astype(np.float32)
    M.quarter_chord(v)
    be = Backend(np.float32)
    stream = Stream()
    be._stream = stream
    verts = DeviceArray.from_numpy(v)
    col = DeviceArray.zeros((3, nc, ns))
    nor = DeviceArray.zeros((3, nc, ns))
    ar = DeviceArray.zeros((nc, ns))
    be.mesh_metrics(0.0, [verts], [col], [nor], [ar])
    wake = np.zeros((4, rows + 1, ns + 1), np.float32)
    te = v[:3, -1, :]
    for r in range(rows + 1):
        wake[0, r] = te[0] + 0.05 * (rows - r)
        wake[1, r] = te[1]
        wake[2, r] = te[2] + 0.02 * math.sin(0.1 * r)
    wake[3] = 1
    dw = DeviceArray.from_numpy(wake)
    gw = DeviceArray.from_numpy(np.random.default_rng(0).standard_normal((rows, ns)).astype(np.float32))
    rhs = DeviceArray.zeros(ns * nc)

    def run(p):
        set_params(p)
        be.rhs_assemble_wake_influence(rhs, [gw], [col], [nor], [dw], [True], rows)
        e0, e1 = Event(), Event()
        e0.record(stream)
        for _ in range(steps):
            be.rhs_assemble_wake_influence(rhs, [gw], [col], [nor], [dw], [True], rows)
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1) / steps

    base = {"wake.waves": defaults()["wake.waves"]}
    best, best_ms, base_ms, tried = _descend(WAKE_SPACE, run, base, repeats)
    out = {"key": key, "params": best, "ms": best_ms, "default_ms": base_ms}
    if persist:
        save(key, best, {"ms": best_ms, "default_ms": base_ms, "tried": tried})
    reset()
    return out


HBVLM_SPACE = [[{"hbvlm.waves": w} for w in (1, 2, 4, 8, 16)],
               [{"hbvlm.min_rows": r} for r in (16, 32, 64, 128)]]


def tune_hbvlm(nc=45, harmonics=5, sets=1, repeats=3, persist=True):
    """Search the HBVLM wake operator's slicing on the 2-DOF section wing
    (nc x 1 panels, `harmonics`), `sets` parameter sets solved together; the
    time of a point is one full run (plan, operator, Anderson, loads)."""
    from . import mesh as M
    from .device import synchronize
    from .hbvlm import HBVLM2
    v = M.rectangular(nc, 1, 1.0, 40000.0)
    hb = HBVLM2("gb300", v)
    hb.init(harmonics, 1.0)
    rng = np.random.default_rng(5)
    dyns = []
    for _ in range(sets):
        d = np.zeros((2, 2 * harmonics + 1))
        d[0, 1:3] = rng.uniform(-0.02, 0.02, 2)
        d[1, 0] = rng.uniform(-0.02, 0.02)
        d[1, 1:3] = rng.uniform(-0.04, 0.04, 2)
        dyns.append(d)
    omegas = [0.4] * sets
    S = hb.parameter_set(0.4, dyns[0])
    cols = hb.plan([S], (0.5,))
    key = hbvlm_key(hb.engine.n, sets * hb.m_coeffs, cols[0]["max_t"], device_sms())

    def run(p):
        hb.gamma_coeffs[:] = 0.0
        forces = [np.zeros((2, 2 * harmonics + 1)) for _ in range(sets)]
        synchronize()
        t0 = time.perf_counter()
        hb._run_sets([hb.parameter_set(o, d) for o, d in zip(omegas, dyns)], (0.5,), forces, False, params=p)
        synchronize()
        return 1000.0 * (time.perf_counter() - t0)

    base = {k: v for k, v in defaults().items() if k.startswith("hbvlm.")}
    best, best_ms, base_ms, tried = _descend(HBVLM_SPACE, run, base, repeats)
    out = {"key": key, "params": best, "ms": best_ms, "default_ms": base_ms}
    if persist:
        save(key, best, {"ms": best_ms, "default_ms": base_ms, "tried": tried})
    reset()
    return out


def main():
    """Tune the benchmark's workloads: the headline batch (512 seeded
    trapezoids x 8 angles, both formulations) and the config-B wake sums
    (20 x 80 wing at several wake lengths), and the HBVLM wake operator of the
    2-DOF section (45 x 1, 5 harmonics; one set, and the 44 sets of a
    finite-difference Jacobian)."""
    from . import mesh as M
    cases = M.batch_cases(512, seed=20261203, n_alpha=8)
    for mode in ("shared", "exact"):
        print(json.dumps(tune_batch(cases, mode=mode, refine=1)))
    print(json.dumps(tune_batch(cases, mode="shared", refine=1, in_flight=2)))
    for rows in (500, 4000, 20000, 40000):
        print(json.dumps(tune_wake((80, 20), rows)))
    for sets in (1, 44):
        print(json.dumps(tune_hbvlm(45, 5, sets)))


if __name__ == "__main__":
    main()
