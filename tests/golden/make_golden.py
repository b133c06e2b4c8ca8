"""Generate the golden fixtures for the steady VLM path.

Run from the repository root:  python -m tests.golden.make_golden
Writes tests/golden/vlm_generated.json (generated planforms) and, when the
reference tree is found (TINYVLM_REF, default /root/reference), vlm_reference_meshes.json
(the reference's own test meshes, read with its plot3d conventions).  Each
case stores the oracle's CL, CDi, CM and a checksum of gamma so later runs
(and the GPU path) can be compared without the reference tree.
"""
import json
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tinyvlm_gb300 import mesh as M  # noqa: E402

REF_MESH = os.path.join(os.environ.get("TINYVLM_REF", "/root/reference"), "mesh")
HERE = os.path.dirname(os.path.abspath(__file__))


def build_case(case):
    """Surfaces (float32, quarter-chord shifted) for a case description."""
    out = []
    for spec in case["meshes"]:
        kind = spec[0]
        if kind == "ref":
            p = os.path.join(REF_MESH, spec[1])
            if not os.path.exists(p):
                return None
            out.append(O.read_plot3d(p))
            continue
        if kind == "elliptic":
            v = M.elliptic(spec[1], spec[2])
        elif kind == "rect":
            v = M.rectangular(spec[1], spec[2], spec[3], spec[4], spec[5])
        elif kind == "trap":
            v = M.trapezoid(spec[1], spec[2], spec[3], spec[4], spec[5])
        else:
            raise ValueError(kind)
        v = v.astype(np.float32)
        M.quarter_chord(v)
        out.append(v)
    return out


def run_cases(cases):
    res = []
    for c in cases:
        surfs = build_case(c)
        if surfs is None:
            continue
        dt = np.float32 if c["precision"] == 32 else np.float64
        r = O.vlm_run([s.astype(dt) for s in surfs], c["alpha"], dtype=dt, ref_pt=c["ref_pt"])
        g = np.concatenate([x.ravel() for x in r["gamma"]]).astype(np.float64)
        d = dict(c)
        d.update(cl=float(r["cl"]), cdi=float(r["cdi"]), cm=[float(x) for x in r["cm"]],
                 gamma_sum=float(g.sum()), gamma_norm=float(np.linalg.norm(g)), n=int(g.size))
        res.append(d)
    return res


def generated_cases():
    cases = []
    for prec in (32, 64):
        for adeg in (0.0, 1.0, 5.0, 10.0):
            a = math.radians(adeg)
            cases.append(dict(name="elliptic16x16_a%g_p%d" % (adeg, prec), meshes=[["elliptic", 16, 16]],
                              alpha=a, precision=prec, ref_pt=[0.0, 0.0, 0.0]))
            cases.append(dict(name="trap8x20_a%g_p%d" % (adeg, prec), meshes=[["trap", 8, 20, 8.0, 0.5, 25.0]],
                              alpha=a, precision=prec, ref_pt=[0.25, 0.0, 0.0]))
            cases.append(dict(name="split2x2_a%g_p%d" % (adeg, prec),
                              meshes=[["rect", 2, 2, 1.0, 20000.0, 0.0], ["rect", 2, 2, 1.0, 20000.0, 20000.0]],
                              alpha=a, precision=prec, ref_pt=[0.0, 0.0, 0.0]))
    return cases


def reference_cases():
    cases = []
    for adeg in (0, 1, 2, 3, 4, 5, 10, 15):
        a = float(np.float32(math.radians(adeg)))
        cases.append(dict(name="ref_elliptic45_a%d" % adeg, meshes=[["ref", "elliptic_45x45.x"]], alpha=a,
                          precision=32, ref_pt=[0.0, 0.0, 0.0]))
        cases.append(dict(name="ref_square_split_a%d" % adeg,
                          meshes=[["ref", "infinite_rectangular_2x2_part0.x"],
                                  ["ref", "infinite_rectangular_2x2_part1.x"]],
                          alpha=a, precision=32, ref_pt=[0.0, 0.0, 0.0]))
    return cases


def main():
    gen = run_cases(generated_cases())
    json.dump({"generator": "tests/golden/make_golden.py", "cases": gen},
              open(os.path.join(HERE, "vlm_generated.json"), "w"), indent=1)
    if os.path.isdir(REF_MESH):
        ref = run_cases(reference_cases())
        json.dump({"generator": "tests/golden/make_golden.py", "cases": ref},
                  open(os.path.join(HERE, "vlm_reference_meshes.json"), "w"), indent=1)
    print("wrote", len(gen), "generated cases")


if __name__ == "__main__":
    main()
