"""UVLM driver on the GPU (time loop on the device) against the oracle's
restatement of UVLM::run, with and without free-wake roll-up."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.kinematics import Assembly, KinematicsTree, rotation_matrix, sin, translation_matrix
from tinyvlm_gb300.uvlm import UVLM, kinematics_arrays

pytestmark = pytest.mark.gpu


def pitch_plunge(k=0.5, h0=0.1, th0=math.radians(3.0), u=1.0):
    tree = KinematicsTree()
    fs = tree.add(lambda t: translation_matrix([-u * t, 0.0, 0.0]))
    heave = tree.add(lambda t: translation_matrix([0.0, 0.0, h0 * sin(k * t)])).after(fs)
    pitch = tree.add(lambda t: rotation_matrix([0.25, 0.0, 0.0], [0.0, 1.0, 0.0],
                                               th0 * sin(k * t + math.pi / 2))).after(heave)
    asm = Assembly(fs)
    asm.add("wing", pitch)
    return asm


def _wing(nc=4, ns=8):
    v = M.rectangular(nc, ns, 1.0, 4.0).astype(np.float32)
    M.quarter_chord(v)
    return v


@pytest.mark.parametrize("rollup", [False, True])
def test_uvlm_double_matches_oracle(cuda, rollup):
    v = _wing()
    asm = pitch_plunge()
    sim = UVLM("gb300", [v], precision=64)
    t_steps = 24
    r = sim.run(asm, t_steps=t_steps, rollup=rollup, return_gamma=True)
    T, Td, fs, ref = kinematics_arrays(asm, t_steps, r["dt"])
    o = O.uvlm_run([v], [True], T, Td, fs, ref, t_steps, r["dt"], dtype=np.float64, rollup=rollup)
    np.testing.assert_allclose(r["cl"][1:-1], o["cl"][1:-1], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(r["cm"][1:-1], o["cm"][1:-1], rtol=1e-9, atol=1e-11)
    g = np.concatenate([x.ravel() for x in o["gamma"]])
    np.testing.assert_allclose(r["gamma"], g, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("rollup", [False, True])
def test_uvlm_float_close_to_double_oracle(cuda, rollup):
    v = _wing(5, 10)
    asm = pitch_plunge()
    sim = UVLM("gb300", [v], precision=32)
    t_steps = 30
    r = sim.run(asm, t_steps=t_steps, rollup=rollup)
    T, Td, fs, ref = kinematics_arrays(asm, t_steps, r["dt"])
    o = O.uvlm_run([v], [True], T, Td, fs, ref, t_steps, r["dt"], dtype=np.float64, rollup=rollup)
    scale = np.abs(o["cl"][1:-1]).max()
    assert np.abs(r["cl"][1:-1] - o["cl"][1:-1]).max() <= 2e-3 * scale


def test_uvlm_two_surfaces_one_non_lifting(cuda):
    a = M.rectangular(3, 4, 0.6, 2.0).astype(np.float32)
    b = M.rectangular(2, 4, 0.4, 2.0).astype(np.float32)
    b[0] += 0.6
    M.quarter_chord(a)
    M.quarter_chord(b)
    asm = pitch_plunge()
    node = asm.surface_kinematics()[0]
    asm2 = Assembly(asm.kinematics())
    asm2.add("wing", node, lifting=False)
    asm2.add("flap", node, lifting=True)
    sim = UVLM("gb300", [a, b], precision=64)
    t_steps = 16
    dt = 0.05
    r = sim.run(asm2, t_steps=t_steps, dt=dt)
    T, Td, fs, ref = kinematics_arrays(asm2, t_steps, dt)
    o = O.uvlm_run([a, b], [False, True], T, Td, fs, ref, t_steps, dt, dtype=np.float64)
    np.testing.assert_allclose(r["cl"][1:-1], o["cl"][1:-1], rtol=1e-9, atol=1e-11)
