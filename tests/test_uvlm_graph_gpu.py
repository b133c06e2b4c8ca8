"""The captured, device-indexed UVLM step (gbvlm_uvlm_step_graph) against the
host-launched step (gbvlm_uvlm_step) and the oracle's float time loop: the
same pitch-plunge run advanced step by step, with the two kinds mixed."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300._lib import GbvlmError, P, PP, call, dims_array
from tinyvlm_gb300.uvlm import kinematics_arrays

from .test_uvlm_gpu import pitch_plunge

pytestmark = pytest.mark.gpu

DT = 0.05


class Stepper:
    def __init__(self, v, T, Td, fs, ref, t_steps, precision=32, rollup=False):
        d = dims_array([(v.shape[2] - 1, v.shape[1] - 1, 0)])
        arr = (ctypes.c_void_p * 1)(v.ctypes.data)
        lf = (ctypes.c_int32 * 1)(1)
        self.h = ctypes.c_void_p()
        call("gbvlm_uvlm_create", ctypes.cast(ctypes.pointer(self.h), P), 1, d, ctypes.cast(arr, PP),
             ctypes.cast(lf, P), int(t_steps), precision)
        self.keep = [np.ascontiguousarray(x) for x in (T, Td, fs, ref)]
        call("gbvlm_uvlm_set_kinematics", self.h, *[ctypes.c_void_p(x.ctypes.data) for x in self.keep])
        call("gbvlm_uvlm_begin", self.h, DT, 1 if rollup else 0, 0.0, None)

    def step(self, graph=False):
        i, cl, cm = ctypes.c_int64(), ctypes.c_double(), (ctypes.c_double * 3)()
        call("gbvlm_uvlm_step_graph" if graph else "gbvlm_uvlm_step", self.h, ctypes.cast(ctypes.pointer(i), P),
             ctypes.cast(ctypes.pointer(cl), P), ctypes.cast(cm, P), None)
        return i.value, cl.value, np.array(cm)

    def __del__(self):
        call("gbvlm_uvlm_destroy", self.h)


def _case(t_steps):
    v = M.rectangular(5, 10, 1.0, 4.0).astype(np.float32)
    M.quarter_chord(v)
    T, Td, fs, ref = kinematics_arrays(pitch_plunge(), t_steps, DT)
    return v, T, Td, fs, ref


def test_graph_steps_match_host_steps_and_oracle(cuda):
    t_steps = 40
    v, T, Td, fs, ref = _case(t_steps)
    a = Stepper(v, T, Td, fs, ref, t_steps)
    b = Stepper(v, T, Td, fs, ref, t_steps)
    host = [a.step() for _ in range(t_steps - 1)]
    # the first step on the host, graph steps, one host step in between, graph steps again
    mixed = [b.step()] + [b.step(graph=True) for _ in range(19)] + [b.step()] + \
        [b.step(graph=True) for _ in range(t_steps - 22)]
    assert [s[0] for s in mixed] == [s[0] for s in host] == list(range(t_steps - 1))
    cl_h = np.array([s[1] for s in host])
    cl_g = np.array([s[1] for s in mixed])
    cm_h = np.array([s[2] for s in host])
    cm_g = np.array([s[2] for s in mixed])
    scale = np.abs(cl_h[1:]).max()
    # the same operator sequence; only the wake sums' split-K grouping differs
    assert np.abs(cl_g[1:] - cl_h[1:]).max() <= 1e-5 * scale
    assert np.abs(cm_g[1:] - cm_h[1:]).max() <= 1e-5 * np.abs(cm_h[1:]).max()
    o = O.uvlm_run([v], [True], T, Td, fs, ref, t_steps, DT, dtype=np.float32)
    assert np.abs(cl_g[1:] - o["cl"][1:t_steps - 1]).max() <= 5e-5 * scale
    # capacity: the last step index is t_steps - 2
    with pytest.raises(GbvlmError, match="wake capacity"):
        b.step(graph=True)


def test_graph_step_refusals(cuda):
    t_steps = 8
    v, T, Td, fs, ref = _case(t_steps)
    s = Stepper(v, T, Td, fs, ref, t_steps)
    with pytest.raises(GbvlmError, match="first step"):
        s.step(graph=True)
    d = Stepper(v, T, Td, fs, ref, t_steps, precision=64)
    d.step()
    with pytest.raises(GbvlmError, match="float runs only"):
        d.step(graph=True)
    r = Stepper(v, T, Td, fs, ref, t_steps, rollup=True)
    r.step()
    with pytest.raises(GbvlmError, match="roll-up"):
        r.step(graph=True)


def _loop(stepper, poll_s=0.02):
    from tinyvlm_gb300.serve import UvlmLoop

    class Sim:
        h = stepper.h
    return UvlmLoop(Sim, poll_s)


def test_request_loop_equals_graph_steps(cuda):
    """The device-resident loop (gbvlm_uvlm_loop_*) takes the same device-indexed step: its results are
    bitwise those of gbvlm_uvlm_step_graph.  Requests submitted back to back run in one graph launch; after
    an idle gap longer than the poll window the loop has ended and the next submit launches it again.
    Submitters on several threads get tickets in one order and the steps follow it.  The wake's capacity
    bounds the tickets, and after the loop is destroyed the case continues from its last step."""
    import threading
    import time
    t_steps = 40
    v, T, Td, fs, ref = _case(t_steps)
    a = Stepper(v, T, Td, fs, ref, t_steps)
    ref_steps = [a.step()] + [a.step(graph=True) for _ in range(t_steps - 2)]
    b = Stepper(v, T, Td, fs, ref, t_steps)
    b.step()
    lp = _loop(b)
    tickets = [lp.submit() for _ in range(10)]
    got = {t: lp.wait(t, 60.0) for t in tickets}
    time.sleep(0.2)  # the loop ends after its 20 ms poll window
    out = {}

    def worker():
        for _ in range(5):
            t = lp.submit()
            out[t] = lp.wait(t, 60.0)
    ths = [threading.Thread(target=worker) for _ in range(3)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    got.update(out)
    st = lp.stats()
    assert st["submitted"] == st["completed"] == 25
    assert 2 <= st["launches"] <= 25
    for t, (i, cl, cm) in got.items():
        ri, rcl, rcm = ref_steps[t]  # ticket t is step t (step 0 was taken on the host)
        assert i == ri == t
        assert cl == rcl and tuple(cm) == tuple(rcm)
    # capacity: t_steps - 2 is the last step index
    for _ in range(t_steps - 2 - 25):
        lp.wait(lp.submit(), 60.0)
    with pytest.raises(GbvlmError, match="wake holds"):
        lp.submit()
    with pytest.raises(GbvlmError, match="request loop"):
        b.step()
    lp.close()
    with pytest.raises(GbvlmError, match="wake capacity"):
        b.step(graph=True)


def test_request_loop_hands_back_to_host_steps(cuda):
    t_steps = 30
    v, T, Td, fs, ref = _case(t_steps)
    a = Stepper(v, T, Td, fs, ref, t_steps)
    ref_steps = [a.step()] + [a.step(graph=True) for _ in range(12)]
    b = Stepper(v, T, Td, fs, ref, t_steps)
    b.step()
    lp = _loop(b)
    for _ in range(6):
        lp.wait(lp.submit(), 60.0)
    lp.close()
    # steps 7.. continue on the host-launched graph from where the loop left the case
    for k in range(7, 13):
        i, cl, cm = b.step(graph=True)
        assert i == k and cl == ref_steps[k][1]
