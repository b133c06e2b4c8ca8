"""Kinematics tree with dual numbers (host side of UVLM/HBVLM)."""
import math

import numpy as np

from tinyvlm_gb300.kinematics import KinematicsTree, rotation_matrix, sin, translation_matrix, Assembly

PI_F = 3.141593


def test_reference_angular_velocity_kat():
    """tests/ut_kinematics.cpp:13-40: pitch 0.5 pi sin(omega t) after a freestream
    translation; angular velocity y = 0.5 pi omega cos(omega t) within 1e-6."""
    u_inf, omega = 1.0, 0.5
    tree = KinematicsTree()
    body = tree.add(lambda t: translation_matrix([0.0, 10.0, 0.0]))
    fs = tree.add(lambda t: translation_matrix([-u_inf * t, 0.0, 0.0])).after(body)
    pitch = tree.add(lambda t: rotation_matrix([0, 0, 0], [0, 1, 0], 0.5 * PI_F * sin(omega * t))).after(fs)
    asm = Assembly(fs)
    asm.add("wing", pitch)
    w = asm.surface_kinematics()[0].angular_velocity(1.0)
    assert abs(w[0]) < 1e-6 and abs(w[2]) < 1e-6
    assert abs(w[1] - 0.5 * PI_F * omega * math.cos(omega * 1.0)) < 1e-6


def test_linear_velocity_matches_finite_difference():
    tree = KinematicsTree()
    fs = tree.add(lambda t: translation_matrix([-t, 0.0, 0.0]))
    heave = tree.add(lambda t: translation_matrix([0.0, 0.0, 0.1 * sin(0.5 * t)])).after(fs)
    pitch = tree.add(lambda t: rotation_matrix([0.25, 0, 0], [0, 1, 0], 0.05 * sin(0.5 * t + 1.0))).after(heave)
    p = (0.7, 1.3, 0.02)
    t, h = 1.7, 1e-6
    v = pitch.linear_velocity(t, p)
    x1 = pitch.transform(t + h) @ np.array([*p, 1.0])
    x0 = pitch.transform(t - h) @ np.array([*p, 1.0])
    np.testing.assert_allclose(v, ((x1 - x0) / (2 * h))[:3], rtol=1e-6, atol=1e-8)
    R = pitch.transform(t)[:3, :3]
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-12)
