"""Loaders for the fixtures the reference's own code wrote
(tests/golden/make_ref_golden.py): its meshes and its drivers' outputs."""
import json
import math
import os

import numpy as np

from tinyvlm_gb300 import mesh as M

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_RUNS = None
_MESHES = None


def runs():
    global _RUNS
    if _RUNS is None:
        with open(os.path.join(GOLDEN, "ref_runs.json")) as f:
            _RUNS = json.load(f)
    return _RUNS


def raw_mesh(name, f64=False):
    """Vertices (4, nc+1, ns+1) as the reference's plot3d reader returns them,
    before the quarter-chord shift."""
    global _MESHES
    if _MESHES is None:
        _MESHES = dict(np.load(os.path.join(GOLDEN, "ref_meshes.npz")))
    xyz = _MESHES[name + ("_f64" if f64 else "")]
    v = np.ones((4,) + xyz.shape[1:], xyz.dtype)
    v[:3] = xyz
    return v


def mesh(name):
    """A reference mesh as VLM::run and UVLM::run see it (quarter-chord shifted, float32)."""
    v = raw_mesh(name)
    M.quarter_chord(v)
    return v


def generated(name):
    """The generated planforms of the VLM fixtures, as the reference read them."""
    if name == "trap8x20":
        v = M.trapezoid(8, 20, 8.0, 0.5, 25.0)
    elif name == "elliptic16x16_generated":
        v = M.elliptic(16, 16)
    elif name == "rect20x80":
        v = M.rectangular(20, 80, 1.0, 4.0)
    else:
        raise KeyError(name)
    v = v.astype(np.float32)
    M.quarter_chord(v)
    return v


VLM_MESHES = {
    "elliptic_16x16": ["elliptic_16x16"],
    "elliptic_45x45": ["elliptic_45x45"],
    "split_2x2": ["infinite_rectangular_2x2_part0", "infinite_rectangular_2x2_part1"],
    "swept_4x4": ["swept_4x4"],
    "rectangular_5x10": ["rectangular_5x10"],
    "trap8x20": None,
    "elliptic16x16_generated": None,
}


def vlm_surfaces(case):
    names = VLM_MESHES[case]
    if names is None:
        return [generated(case)]
    return [mesh(n) for n in names]


def pitch_plunge_assembly(p):
    """The pitch-plunge motion of the UVLM fixture (oracle/ref/ref_fixtures.cpp cmd_uvlm)."""
    from tinyvlm_gb300.kinematics import Assembly, KinematicsTree, rotation_matrix, sin, translation_matrix
    k, h = p["k"], p["heave"]
    amp, ph = math.radians(p["pitch_deg"]), math.radians(p["phase_deg"])
    tree = KinematicsTree()
    fs = tree.add(lambda t: translation_matrix([-t, 0.0, 0.0]))
    heave = tree.add(lambda t: translation_matrix([0.0, 0.0, h * sin(k * t)])).after(fs)
    pitch = tree.add(lambda t: rotation_matrix([0.25, 0, 0], [0, 1, 0], amp * sin(ph + k * t))).after(heave)
    asm = Assembly(fs)
    asm.add("wing", pitch)
    return asm


def theodorsen_assembly(k=0.25):
    """tests/uvlm_theodorsen.cpp:19-66: pitch 1 deg (sin wt + 2 sin 3wt) about the quarter chord,
    w = k u / b with b = 0.5, u = 1."""
    from tinyvlm_gb300.kinematics import Assembly, KinematicsTree, rotation_matrix, sin, translation_matrix
    omega = k * 1.0 / 0.5
    amp = math.radians(1.0)
    tree = KinematicsTree()
    fs = tree.add(lambda t: translation_matrix([-t, 0.0, 0.0]))
    pitch = tree.add(lambda t: rotation_matrix([0.25, 0, 0], [0, 1, 0],
                                               amp * (sin(omega * t) + 2.0 * sin(3.0 * omega * t)))).after(fs)
    asm = Assembly(fs)
    asm.add("wing", pitch)
    return asm


def reference_time_steps(v, t_final, speed=1.0):
    """UVLM::run's step count and time step in float (vlm.cpp:379-387)."""
    d = v[:3, -1, 0].astype(np.float32) - v[:3, -2, 0].astype(np.float32)
    chord = np.float32(math.sqrt(float(np.float32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))))
    dt = np.float32(chord / np.float32(speed))
    return int(np.float32(t_final) / dt), float(dt)


def hbvlm3_meshes(case):
    return [raw_mesh(case["wing"][:-2], f64=True), raw_mesh(case["flap"][:-2], f64=True)]


def cl_rel_err(got, want, scale):
    """|got - want| / max(|want|, 1e-3 * scale): relative, guarded near zero lift."""
    return abs(got - want) / max(abs(want), 1e-3 * scale)
