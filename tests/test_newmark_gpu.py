"""Device Newmark-beta (gbvlm_newmark_*, double) against the golden vectors
of the reference's scripts/newmark.py on the 3-DOF system of its
tests/newmark.cpp, and against the oracle on a forced non-symmetric case."""
import json
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tinyvlm_gb300.integrator import NewmarkBeta

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "newmark_3dof.json")


def _cm(x):  # (n, n) device tensor whose memory is x in column-major order
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, np.float64).T)).cuda()


def _drive(M, C, K, u0, v0, dt, steps, loads=None):
    n = len(u0)
    Md, Cd, Kd = _cm(M), _cm(C), _cm(K)
    nb = NewmarkBeta()
    nb.init(Md, Cd, Kd, dt)
    u = torch.zeros((steps + 1, n), dtype=torch.float64, device="cuda")
    v = torch.zeros_like(u)
    a = torch.zeros_like(u)
    u[0] = torch.tensor(u0, dtype=torch.float64)
    v[0] = torch.tensor(v0, dtype=torch.float64)
    a[0] = torch.tensor(np.linalg.solve(M, -np.asarray(C) @ np.asarray(v0) - np.asarray(K) @ np.asarray(u0)))
    du, dv, da = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3))
    dF = torch.zeros(n, dtype=torch.float64, device="cuda")
    for i in range(steps):
        if loads is not None:
            dF.copy_(torch.from_numpy(loads[i + 1] - loads[i]))
        vi, ai = v[i].contiguous(), a[i].contiguous()
        nb.step(Md, Cd, vi, ai, du, dv, da, dF, dt)
        u[i + 1] = u[i] + du
        v[i + 1] = v[i] + dv
        a[i + 1] = a[i] + da
    torch.cuda.synchronize()
    return u.cpu().numpy(), v.cpu().numpy(), a.cpu().numpy()


def test_newmark_3dof_against_reference_script(cuda):
    with open(GOLD) as f:
        g = json.load(f)
    u, v, a = _drive(np.array(g["M"]), np.array(g["C"]), np.array(g["K"]), g["u0"], g["v0"], g["dt"], g["steps"])
    for name, x in (("u", u), ("v", v), ("a", a)):
        ref = np.array(g[name])
        assert np.abs(x - ref).max() <= 1e-11 * max(1.0, np.abs(ref).max()), name


def test_newmark_forced_nonsymmetric_against_oracle(cuda):
    rng = np.random.default_rng(4)
    n = 4
    M = np.eye(n) + 0.1 * rng.standard_normal((n, n))
    C = 0.05 * rng.standard_normal((n, n))
    K = 3.0 * np.eye(n) + 0.3 * rng.standard_normal((n, n))
    dt, steps = 0.02, 300
    t = np.arange(steps + 1) * dt
    loads = np.stack([np.sin((q + 1) * t) for q in range(n)], axis=1)
    u, v, a = _drive(M, C, K, np.zeros(n), np.ones(n), dt, steps, loads)
    Ke = O.newmark_keff(M, C, K, dt)
    uo = np.zeros((steps + 1, n))
    vo = np.zeros_like(uo)
    ao = np.zeros_like(uo)
    vo[0] = 1.0
    ao[0] = np.linalg.solve(M, -C @ vo[0] - K @ uo[0])
    for i in range(steps):
        du, dv, da = O.newmark_step(M, C, Ke, vo[i], ao[i], loads[i + 1] - loads[i], dt)
        uo[i + 1], vo[i + 1], ao[i + 1] = uo[i] + du, vo[i] + dv, ao[i] + da
    assert np.abs(u - uo).max() <= 1e-10 * np.abs(uo).max()
    assert np.abs(v - vo).max() <= 1e-10 * np.abs(vo).max()
