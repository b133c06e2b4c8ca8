"""Golden vectors of the Newmark-beta integrator from the reference's own
Python implementation (scripts/newmark.py, numpy only).

Run from the repository root with the reference tree at TINYVLM_REF
(default /root/reference):  python -m tests.golden.make_newmark_golden
Writes tests/golden/newmark_3dof.json: the 3-DOF free response that the
reference's tests/newmark.cpp integrates (M = I, its C and K, u0 = 0,
v0 = 1, dt = 0.1, t = 0..20), stepped with scripts/newmark.py's
newmark_beta_step exactly as tests/newmark.cpp drives NewmarkBeta::step.
"""
import importlib.util
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SCRIPT = os.path.join(os.environ.get("TINYVLM_REF", "/root/reference"), "scripts", "newmark.py")

# the system of tests/newmark.cpp:66-92 (column-major there; symmetric here)
K = np.array([[400.0, -200.0, 0.0], [-200.0, 400.0, -200.0], [0.0, -200.0, 200.0]])
C = np.array([[0.55, -0.2, 0.0], [-0.2, 0.4, -0.2], [0.0, -0.2, 0.35]])
M = np.eye(3)
DT, T_FINAL = 0.1, 20.0


def main():
    spec = importlib.util.spec_from_file_location("ref_newmark", SCRIPT)
    ref = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref)
    steps = int(T_FINAL / DT)
    u = np.zeros((steps + 1, 3))
    v = np.zeros((steps + 1, 3))
    a = np.zeros((steps + 1, 3))
    v[0] = 1.0
    a[0] = np.linalg.solve(M, -C @ v[0] - K @ u[0])
    for i in range(steps):
        du, dv, da = ref.newmark_beta_step(M, C, K, v[i], a[i], np.zeros(3), DT)
        u[i + 1], v[i + 1], a[i + 1] = u[i] + du, v[i] + dv, a[i] + da
    out = {"source": "scripts/newmark.py newmark_beta_step on the system of tests/newmark.cpp",
           "M": M.tolist(), "C": C.tolist(), "K": K.tolist(), "dt": DT, "steps": steps,
           "u0": [0.0, 0.0, 0.0], "v0": [1.0, 1.0, 1.0],
           "u": u.tolist(), "v": v.tolist(), "a": a.tolist()}
    with open(os.path.join(HERE, "newmark_3dof.json"), "w") as f:
        json.dump(out, f)
    print("wrote newmark_3dof.json, %d steps, max |u| %.4f" % (steps, np.abs(u).max()))


if __name__ == "__main__":
    main()
