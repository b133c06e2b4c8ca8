"""The GPU paths against outputs of the reference's own code.

tests/golden/ref_runs.json holds what the reference's VLM::run, UVLM::run
and libhbvlm3 HBVLM.run computed, compiled unmodified on the CPU
(tests/golden/make_ref_golden.py); tests/test_ref_parity.py pins the oracle
to the same outputs.  Here:

  * VLM (config A exactly: the reference's mesh/elliptic_16x16.x, read back
    through the library's plot3d reader gbvlm_read_plot3d): the double path
    equals the oracle's double solve to 1e-9; the float path (the
    reference's semantics) is at least as close to that exact solve as the
    reference's own float path, whose CL is 5e-6 to 5e-5 from it; the
    batched mixed-precision path in exact mode (the reference's
    alpha-dependent system) is within 1e-5 of it in CL;
  * UVLM: the float device time loop reproduces the reference's CL(t)
    records, 20 x 80 pitch-plunge and the reference's Theodorsen run;
  * HBVLM: forces_t of the reference's libhbvlm3 within 1e-9.
"""
import math
import os
import tempfile
import types

import numpy as np
import pytest

from oracle import oracle as O
from tests import ref_fixtures as R
from tinyvlm_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _exact(surfs, alpha):
    return O.vlm_run([s.astype(np.float64) for s in surfs], float(np.float32(alpha)), dtype=np.float64)


def _flat(gs):
    return np.concatenate([np.asarray(g, np.float64).ravel() for g in gs])


def _check_case(case, surfs_or_paths, surfs):
    from tinyvlm_gb300.vlm import VLM, FlowData
    cases = R.runs()["vlm"][case]
    exact = [_exact(surfs, c["alpha"]) for c in cases]
    ref_err = max(R.cl_rel_err(c["cl"], float(e["cl"]), 1.0) for c, e in zip(cases, exact))
    v32 = VLM("gb300", surfs_or_paths, precision=32)
    v64 = VLM("gb300", surfs_or_paths, precision=64)
    worst32 = 0.0
    for c, e in zip(cases, exact):
        al = float(np.float32(c["alpha"]))
        r64, g64 = v64.run(FlowData(al), return_gamma=True)
        assert R.cl_rel_err(r64.cl, float(e["cl"]), 1.0) <= 1e-9, (case, c["alpha_deg"], r64.cl, float(e["cl"]))
        r32 = v32.run(FlowData(al))
        err32 = R.cl_rel_err(r32.cl, float(e["cl"]), 1.0)
        worst32 = max(worst32, err32)
        # float against the reference's float result: within both float paths' distance to the exact solve
        assert R.cl_rel_err(r32.cl, c["cl"], 1.0) <= 3 * ref_err + 2e-6, (case, c["alpha_deg"], r32.cl, c["cl"])
        if "gamma" in c:
            g_ref = _flat(c["gamma"])
            scale = np.abs(g_ref).max()
            if scale > 0:
                assert np.abs(g64 - _flat(e["gamma"])).max() <= 1e-9 * scale, (case, c["alpha_deg"])
    print(case, "reference float CL error %.2e, GPU float %.2e" % (ref_err, worst32))
    assert worst32 <= 2 * ref_err + 2e-6, (case, worst32, ref_err)
    return exact


def test_config_a_elliptic_16x16_through_the_plot3d_reader(cuda):
    """Config A exactly: the reference's mesh/elliptic_16x16.x (written back from the reference reader's
    numbers), alpha in {0,1,2,3,4,5,10,15} deg, through VLM("gb300", [path])."""
    from tinyvlm_gb300.vlm import read_plot3d
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "elliptic_16x16.x")
        M.write_plot3d(path, R.raw_mesh("elliptic_16x16"))
        assert np.array_equal(read_plot3d(path), R.mesh("elliptic_16x16"))  # gbvlm_read_plot3d, shift included
        _check_case("elliptic_16x16", [path], [R.mesh("elliptic_16x16")])


@pytest.mark.parametrize("case", ["elliptic_45x45", "split_2x2", "swept_4x4", "rectangular_5x10", "trap8x20",
                                  "elliptic16x16_generated"])
def test_vlm_reference_meshes(cuda, case):
    surfs = R.vlm_surfaces(case)
    _check_case(case, surfs, surfs)


@pytest.mark.parametrize("case", ["elliptic_16x16", "elliptic_45x45", "swept_4x4", "trap8x20"])
def test_batched_exact_mode_on_reference_meshes(cuda, case):
    """The headline batched mixed-precision path, exact (alpha-dependent) mode = VLM::run's system: CL within
    1e-5 of the exact solve for every alpha of the reference's run."""
    from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts
    v = R.vlm_surfaces(case)[0]
    cases = R.runs()["vlm"][case]
    alphas = [float(np.float32(c["alpha"])) for c in cases]
    cobj = types.SimpleNamespace(verts=v, ns=v.shape[2] - 1, nc=v.shape[1] - 1, alphas=alphas)
    bs = BatchSolver([cobj], mode="exact", refine=1)
    bs.set_inputs(pack_verts([cobj]), pack_alphas([cobj]))
    bs.run()
    co, _ = bs.results()
    for k, a in enumerate(alphas):
        e = _exact([v], a)
        err = R.cl_rel_err(co[k, 0], float(e["cl"]), 1.0)
        assert err <= 1e-5, (case, a, co[k, 0], float(e["cl"]))
        assert R.cl_rel_err(co[k, 0], cases[k]["cl"], 1.0) <= 1e-4


def _uvlm(v, asm, t_steps, dt, precision=32):
    from tinyvlm_gb300.uvlm import UVLM
    return UVLM("gb300", [v], precision=precision).run(asm, t_steps=t_steps, dt=dt)


def test_uvlm_pitch_plunge_matches_reference_run(cuda):
    """UVLM::run on the 20 x 80 pitch-plunge rectangle (BASELINE config B's wing and motion): every
    recorded CL(t) within 2e-5 of max |CL| of the reference's float run; the double device path within
    2e-5 too (the reference's float error)."""
    d = R.runs()["uvlm"]["pitch_plunge_20x80"]
    v = R.generated("rect20x80")
    t_steps, dt = R.reference_time_steps(v, d["params"]["t_final"])
    asm = R.pitch_plunge_assembly(d["params"])
    cl_ref = np.asarray(d["cl"])
    scale = np.abs(cl_ref).max()
    for prec in (32, 64):
        out = _uvlm(v, asm, t_steps, dt, prec)
        err = np.abs(out["cl"][1:t_steps - 1] - cl_ref) / scale
        print("pitch-plunge precision %d: max |dCL|/max|CL| %.2e" % (prec, err.max()))
        assert err.max() <= 2e-5, (prec, err.max())


def test_uvlm_theodorsen_matches_reference_run(cuda):
    """The reference's own tests/uvlm_theodorsen.cpp run, all 148 recorded steps, float device loop."""
    d = R.runs()["uvlm"]["theodorsen_5x100"]
    v = R.mesh("infinite_rectangular_5x100")
    t_final = 3.0 * 2.0 * math.pi / (d["k"] * 1.0 / 0.5)
    t_steps, dt = R.reference_time_steps(v, t_final)
    out = _uvlm(v, R.theodorsen_assembly(d["k"]), t_steps, dt)
    cl_ref = np.asarray(d["cl"])
    err = np.abs(out["cl"][1:t_steps - 1] - cl_ref) / np.abs(cl_ref).max()
    print("theodorsen: max |dCL|/max|CL| %.2e" % err.max())
    assert err.max() <= 2e-5, err.max()


@pytest.mark.parametrize("idx", [0, 1])
def test_hbvlm3_matches_reference_libhbvlm3(cuda, idx):
    from tinyvlm_gb300.hbvlm import HBVLM3
    c = R.runs()["hbvlm3"][idx]
    hb = HBVLM3("gb300", R.hbvlm3_meshes(c))
    hb.init(c["harmonics"], c["scaling"])
    ft = np.zeros((3, 2 * c["harmonics"] + 1))
    hb.run(c["omega"], c["U"], np.asarray(c["dyn_f"]), ft)
    ref = np.asarray(c["forces_t"])
    err = np.abs(ft - ref).max() / np.abs(ref).max()
    print("hbvlm3 case %d: max rel err %.2e (%d Anderson iterations)" % (idx, err, hb.iterations))
    assert err <= 1e-9, err
