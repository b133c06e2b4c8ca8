"""The oracle against outputs of the reference's own code (CPU).

tests/golden/ref_runs.json was written by the reference's drivers, CPU
backend, pybind module and test programs, compiled unmodified from the
reference tree over the oracle's C restatement of the four ISPC kernels
(oracle/ref/build_ref.py, tests/golden/make_ref_golden.py).  These tests pin
the oracle's restatement of the drivers (oracle/oracle.py: VLM::run,
UVLM::run, HBVLM::run) and the package's plot3d reader to that code.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from tests import ref_fixtures as R
from tinyvlm_gb300 import mesh as M


def test_reference_programs_pass_their_known_answers():
    """The reference's tests/*.cpp (elliptic lifting line 3 %, 2 pi alpha 1 % incl. the two-surface split,
    NLVLM curves 1 %, kinematics, tensor strides, Newmark) exit 0 when built over the restated kernels."""
    progs = R.runs()["programs"]
    for name in ("vlm_elliptic_coeffs", "vlm_square_coeffs", "nlvlm_curves", "ut_kinematics", "ut_tensor", "newmark"):
        assert progs[name]["returncode"] == 0, name
    table = dict((a, cl) for a, cl in progs["vlm_elliptic_coeffs"]["cl_table"])
    assert abs(table[5.0] - 0.465258) < 1e-6


@pytest.mark.parametrize("case", sorted(R.VLM_MESHES))
def test_oracle_vlm_run_matches_reference_run(case):
    """VLM::run (vlm/src/vlm.cpp:97-151): the oracle's float restatement gives the reference's CL and
    circulation to within float rounding (the only difference is the order of the ISPC lane sums)."""
    surfs = R.vlm_surfaces(case)
    for c in R.runs()["vlm"][case]:
        r = O.vlm_run(surfs, np.float32(c["alpha"]))
        assert abs(float(r["cl"]) - c["cl"]) <= 2e-6 * max(abs(c["cl"]), 1e-2), (case, c["alpha_deg"])
        if "gamma" in c:
            for g_ref, g in zip(c["gamma"], r["gamma"]):
                g_ref = np.asarray(g_ref)
                assert np.abs(np.asarray(g).ravel() - g_ref).max() <= 2e-6 * max(np.abs(g_ref).max(), 1e-30)


def test_plot3d_reader_matches_reference_reader():
    """mesh.read_plot3d (vlm/src/vlm_mesh.cpp:16-92): a reference mesh written back out and read gives the
    reference reader's vertices, quarter-chord shift included, bit for bit."""
    import tempfile, os
    for name in ("elliptic_16x16", "swept_4x4", "infinite_rectangular_2x2_part1"):
        raw = R.raw_mesh(name)
        with tempfile.TemporaryDirectory() as d:
            p = os.path.join(d, name + ".x")
            M.write_plot3d(p, raw)
            assert np.array_equal(M.read_plot3d(p, qc=False), raw)
            assert np.array_equal(M.read_plot3d(p), R.mesh(name))


def _uvlm_oracle(v, asm, t_steps, dt, dtype=np.float32):
    from tinyvlm_gb300.uvlm import kinematics_arrays
    T, Td, fs, ref = kinematics_arrays(asm, t_steps, dt)
    return O.uvlm_run([v], [True], T, Td, fs, ref, t_steps, dt, dtype=dtype)


def test_oracle_uvlm_run_matches_reference_pitch_plunge():
    """UVLM::run (vlm/src/vlm.cpp:358-509) on the 20 x 80 pitch-plunge rectangle: CL(t) of every recorded
    step.  The reference evaluates the kinematics in float dual numbers, the oracle in double."""
    d = R.runs()["uvlm"]["pitch_plunge_20x80"]
    p = d["params"]
    v = R.generated("rect20x80")
    t_steps, dt = R.reference_time_steps(v, p["t_final"])
    assert t_steps - 2 == len(d["cl"])
    out = _uvlm_oracle(v, R.pitch_plunge_assembly(p), t_steps, dt)
    cl_ref = np.asarray(d["cl"])
    scale = np.abs(cl_ref).max()
    err = np.abs(out["cl"][1:t_steps - 1] - cl_ref) / scale
    assert err.max() <= 2e-5, err.max()
    np.testing.assert_allclose(np.arange(1, t_steps - 1) * np.float32(dt), d["t"], rtol=1e-6, atol=1e-6)


def test_oracle_uvlm_run_matches_reference_theodorsen():
    """The reference's own tests/uvlm_theodorsen.cpp run (infinite_rectangular_5x100, k = 0.25): its
    recorded CL(t), first 60 steps."""
    d = R.runs()["uvlm"]["theodorsen_5x100"]
    v = R.mesh("infinite_rectangular_5x100")
    k = d["k"]
    t_final = 3.0 * 2.0 * math.pi / (k * 1.0 / 0.5)
    t_steps, dt = R.reference_time_steps(v, t_final)
    assert t_steps - 2 == len(d["cl"])
    steps = 62
    out = _uvlm_oracle(v, R.theodorsen_assembly(k), steps, dt)
    cl_ref = np.asarray(d["cl"][:steps - 2])
    err = np.abs(out["cl"][1:steps - 1] - cl_ref) / np.abs(np.asarray(d["cl"])).max()
    assert err.max() <= 2e-5, err.max()


@pytest.mark.parametrize("idx", [0, 1])
def test_oracle_hbvlm_run_matches_reference_libhbvlm3(idx):
    """lib/libhbvlm3.cpp HBVLM.run (3-DOF wing + flap): the oracle's restatement of HBVLM::run on the
    package's host-side plan (time step, instances, kinematics, DFT) gives the reference's forces_t."""
    from tinyvlm_gb300.hbvlm import HBVLM3
    c = R.runs()["hbvlm3"][idx]
    hb = HBVLM3("gb300", R.hbvlm3_meshes(c))
    hb.init(c["harmonics"], c["scaling"])
    dyn = np.asarray(c["dyn_f"])
    L = hb.plan([hb.parameter_set(c["omega"], c["U"], dyn)], hb._refs())[0]
    x0 = np.zeros_like(hb.gamma_coeffs)
    _, out, _ = O.hbvlm_run(hb.verts, [False, True], c["harmonics"], c["omega"], L["dt"], L["max_t"], L["wake_T"],
                            L["inst"], L["dft"], L["ddft"], L["force_inst"], L["fs"], L["ref_a"], L["ref_b"], True,
                            x0, 1e-12)
    ref = np.asarray(c["forces_t"])
    scale = np.abs(ref).max()
    err = np.abs(out[:3] - ref).max() / scale
    print("hbvlm3 case", idx, "max rel err", err)
    assert err <= 1e-9, err
