"""Golden fixtures written by the reference's own code, compiled here.

Run from the repository root:  python -m tests.golden.make_ref_golden

Needs the reference tree (TINYVLM_REF, default /root/reference).  It builds
oracle/_ref with oracle/ref/build_ref.py: the reference's drivers, CPU
backend, pybind module and test programs, compiled unmodified, over the
oracle's C restatement of the four ISPC kernels.  It then writes:

  tests/golden/ref_meshes.npz   the reference meshes the tests use, as the
                                reference's plot3d reader returns them before
                                the quarter-chord shift (float32, (3, nc+1, ns+1));
                                the harmonic-balance meshes also in float64
                                ("<name>_f64"), as lib/libhbvlm3.cpp reads them
  tests/golden/ref_runs.json    what the reference's code computes:
     vlm        VLM::run (vlm/src/vlm.cpp:97-151): CL and circulation per alpha
     uvlm       UVLM::run (vlm/src/vlm.cpp:358-509): the CL(t) record it writes
                and the last circulation, for a pitch-plunge rectangle and
                for the reference's own tests/uvlm_theodorsen.cpp run
     hbvlm3     lib/libhbvlm3.cpp HBVLM.run: forces_t for seeded motions
     programs   exit status and printed CL tables of the reference's test
                programs (tests/*.cpp), which assert their own known answers

The generated planforms are written to plot3d files with
tinyvlm_gb300.mesh.write_plot3d and read by the reference's reader, like the
reference meshes.
"""
import json
import math
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.ref import build_ref  # noqa: E402
from tinyvlm_gb300 import mesh as M  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ALPHAS = [0, 1, 2, 3, 4, 5, 10, 15]

REF_MESHES = ["elliptic_16x16.x", "elliptic_45x45.x", "elliptic_128x128.x", "infinite_rectangular_2x2_part0.x",
              "infinite_rectangular_2x2_part1.x", "infinite_rectangular_2x4.x", "infinite_rectangular_10x5.x",
              "infinite_rectangular_20x5.x", "swept_4x4.x", "rectangular_5x10.x", "infinite_rectangular_5x100.x",
              "infinite_rectangular_5x200.x", "3dof_wing_9x5.x", "3dof_flap_3x5.x", "3dof_wing_45x1.x",
              "3dof_flap_15x1.x"]

# BASELINE config B's motion at a prefix the reference's float CPU path finishes quickly
PITCH_PLUNGE = dict(nc=20, ns=80, chord=1.0, semispan=4.0, t_final=2.0, k=0.5, heave=0.1, pitch_deg=3.0,
                    phase_deg=90.0)


def _prog(name):
    return os.path.join(build_ref.OUT, name)


def _last_json(out):
    return json.loads(out.strip().splitlines()[-1])


def _run(args, cwd=None):
    r = subprocess.run(args, capture_output=True, text=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError("%s failed (%d):\n%s\n%s" % (args, r.returncode, r.stdout[-2000:], r.stderr[-2000:]))
    return r.stdout


def ref_mesh(name, qc):
    d = _last_json(_run([_prog("ref_fixtures"), "mesh", os.path.join(build_ref.REF, "mesh", name), "1" if qc else "0"]))
    ns, nc = d["ns"], d["nc"]
    return np.asarray(d["xyz"], np.float32).reshape(3, nc + 1, ns + 1)


def vlm_cases(tmp):
    trap = os.path.join(tmp, "trap8x20.x")
    M.write_plot3d(trap, M.trapezoid(8, 20, 8.0, 0.5, 25.0))
    ell = os.path.join(tmp, "elliptic16x16_generated.x")
    M.write_plot3d(ell, M.elliptic(16, 16))
    mesh = lambda n: os.path.join(build_ref.REF, "mesh", n)
    cases = [
        ("elliptic_16x16", [mesh("elliptic_16x16.x")], ALPHAS, True),
        ("elliptic_45x45", [mesh("elliptic_45x45.x")], ALPHAS, False),
        ("split_2x2", [mesh("infinite_rectangular_2x2_part0.x"), mesh("infinite_rectangular_2x2_part1.x")], ALPHAS,
         True),
        ("swept_4x4", [mesh("swept_4x4.x")], ALPHAS, True),
        ("rectangular_5x10", [mesh("rectangular_5x10.x")], [0, 5, 10], True),
        ("trap8x20", [trap], [0, 1, 5, 10], True),
        ("elliptic16x16_generated", [ell], [0, 5, 10], True),
    ]
    out = {}
    for name, meshes, alphas, keep_gamma in cases:
        d = _last_json(_run([_prog("ref_fixtures"), "vlm", ",".join(str(a) for a in alphas)] + meshes))
        for c in d["cases"]:
            if not keep_gamma and c["alpha_deg"] != 5:
                c.pop("gamma")
        out[name] = d["cases"]
        print("vlm", name, [round(c["cl"], 6) for c in d["cases"]])
    return out


def uvlm_cases(tmp):
    p = PITCH_PLUNGE
    path = os.path.join(tmp, "rect20x80.x")
    M.write_plot3d(path, M.rectangular(p["nc"], p["ns"], p["chord"], p["semispan"]))
    d = _last_json(_run([_prog("ref_fixtures"), "uvlm", path, repr(p["t_final"]), repr(p["k"]), repr(p["heave"]),
                         repr(p["pitch_deg"]), repr(p["phase_deg"])], cwd=tmp))
    d["params"] = p
    print("uvlm pitch-plunge: %d records" % len(d["cl"]))
    # the reference's own test program (tests/uvlm_theodorsen.cpp: infinite_rectangular_5x100, pitch
    # 1 deg (sin wt + 2 sin 3wt) about the quarter chord, k = 0.25, three cycles) writes cl_data_CPU.txt
    cwd = build_ref.test_cwd()
    _run([_prog("uvlm_theodorsen")], cwd=cwd)
    rows = [list(map(float, ln.split())) for ln in open(os.path.join(cwd, "cl_data_CPU.txt")).read().splitlines()[1:]
            if ln.strip()]
    theo = dict(mesh="infinite_rectangular_5x100.x", k=0.25, t=[r[0] for r in rows], z=[r[1] for r in rows],
                cl=[r[2] for r in rows], pitch=[r[3] for r in rows])
    print("uvlm theodorsen: %d records" % len(rows))
    return {"pitch_plunge_20x80": d, "theodorsen_5x100": theo}


def hbvlm3_cases(tmp):
    sys.path.insert(0, build_ref.OUT)
    import libhbvlm3  # the reference's pybind module, built in oracle/_ref
    out = []
    for wing_name, flap_name, H, omega, U, seed in (("3dof_wing_9x5.x", "3dof_flap_3x5.x", 2, 1.0, 10.0, 1),
                                                   ("3dof_wing_45x1.x", "3dof_flap_15x1.x", 3, 0.8, 12.0, 2)):
        rng = np.random.default_rng(seed)
        dyn = np.zeros((3, 2 * H + 1))
        dyn[:, 1:3] = 0.02 * rng.standard_normal((3, 2))
        dyn[1, 0] = 0.01
        ft = np.zeros((3, 2 * H + 1))
        hb = libhbvlm3.HBVLM("cpu", [os.path.join(build_ref.REF, "mesh", wing_name),
                                     os.path.join(build_ref.REF, "mesh", flap_name)])
        hb.init(H, 1.0 / 0.127)
        hb.run(omega, U, dyn, ft)
        out.append(dict(wing=wing_name, flap=flap_name, harmonics=H, scaling=1.0 / 0.127, omega=omega, U=U,
                        dyn_f=dyn.tolist(), forces_t=ft.tolist()))
        print("hbvlm3", wing_name, flap_name, "forces_t[0]", np.round(ft[0], 6))
    return out


def _table(text):
    """Rows (alpha_deg, CL) of the tables the reference's VLM tests print."""
    rows = []
    for ln in text.splitlines():
        m = re.match(r"\|\s*(-?[\d.]+)\s*\|\s*(-?[\d.]+)\s*\|", ln)
        if m:
            rows.append([float(m.group(1)), float(m.group(2))])
    return rows


def programs():
    out = {}
    cwd = build_ref.test_cwd()
    for t in build_ref.TESTS:
        if t == "uvlm_theodorsen":
            continue
        r = subprocess.run([_prog(t)], capture_output=True, text=True, cwd=cwd)
        out[t] = dict(returncode=r.returncode, cl_table=_table(r.stdout))
        print("program", t, "rc", r.returncode)
    return out


def main():
    build_ref.build()
    meshes = {n[:-2]: ref_mesh(n, False) for n in REF_MESHES}
    for n in REF_MESHES:  # our reader + shift reproduces the reference's reader bit for bit
        v = np.ones((4,) + meshes[n[:-2]].shape[1:], np.float32)
        v[:3] = meshes[n[:-2]]
        M.quarter_chord(v)
        assert np.array_equal(v[:3], ref_mesh(n, True)), n
    for n in REF_MESHES:
        if n.startswith("3dof_"):  # libhbvlm3 parses its meshes into doubles (strtod rounding, as float())
            meshes[n[:-2] + "_f64"] = M.read_plot3d(os.path.join(build_ref.REF, "mesh", n), qc=False,
                                                    dtype=np.float64)[:3]
    np.savez_compressed(os.path.join(HERE, "ref_meshes.npz"), **meshes)
    with tempfile.TemporaryDirectory() as tmp:
        runs = dict(generator="tests/golden/make_ref_golden.py", vlm=vlm_cases(tmp), uvlm=uvlm_cases(tmp),
                    hbvlm3=hbvlm3_cases(tmp), programs=programs())
    with open(os.path.join(HERE, "ref_runs.json"), "w") as f:
        json.dump(runs, f, separators=(",", ":"))
    print("wrote ref_meshes.npz and ref_runs.json")


if __name__ == "__main__":
    main()
