"""Served mixed stream: steady, UVLM-step and HBVLM requests with continuous
batching across lanes give the same result alone and in the mix."""
import numpy as np
import pytest

from tinyvlm_gb300 import serve as S

pytestmark = pytest.mark.gpu


def _requests(seed=4):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(24):
        k = i % 3
        if k == 0:
            reqs.append(("steady", (S.steady_case(rng, 64, 600),)))
        elif k == 1:
            reqs.append(("uvlm", None))
        else:
            reqs.append(("hbvlm", S.hbvlm_request(rng, harmonics=2)))
    return reqs


def _serve(reqs, lanes, concurrent):
    srv = S.Server(lanes=lanes, hbm_budget=4 << 30, max_batch=16,
                   uvlm=S.resident_uvlm(ns=8, nc=4, warm_steps=10, capacity=64),
                   hbvlm=S.hbvlm_factory(nc=10, harmonics=2)).start()
    out = []
    for rid, (kind, payload) in enumerate(reqs):
        r = srv.submit(S.Request(rid, kind, payload))
        if not concurrent:
            r.done.wait()
        out.append(r)
    for r in out:
        r.done.wait()
    srv.shutdown()
    for r in out:
        assert r.error is None, r.error
    return out, srv


def test_alone_equals_mix(cuda):
    reqs = _requests()
    alone, _ = _serve(reqs, lanes=1, concurrent=False)
    mix, srv = _serve(reqs, lanes=3, concurrent=True)
    for a, b in zip(alone, mix):
        if a.kind == "uvlm":
            assert a.result[0] == b.result[0]
            np.testing.assert_allclose(a.result[1:2], b.result[1:2], rtol=1e-6, atol=1e-9)
        else:
            np.testing.assert_allclose(a.result, b.result, rtol=1e-9, atol=1e-12)
    # continuous batching actually grouped steady requests in the concurrent run
    assert srv.stats["steady_groups"] <= 8


def test_budget_admission_blocks_until_free(cuda):
    srv = S.Server(lanes=2, hbm_budget=S.steady_bytes(400) + 1, max_batch=8).start()
    rng = np.random.default_rng(1)
    reqs = [srv.submit(S.Request(i, "steady", (S.steady_case(rng, 300, 400),))) for i in range(4)]
    for r in reqs:
        assert r.done.wait(60)
        assert r.error is None
    srv.shutdown()
    assert srv.used == 0


def test_served_results_match_the_oracle(cuda):
    """Every result of a concurrent mixed run against the oracle: steady CL and CM (exact formulation, one
    refinement sweep) within 1e-5 of the double solve; each UVLM step's CL within 2e-5 of max |CL| of the
    oracle's float time loop at the same step; each HBVLM residual's forces within 1e-7 of the oracle's
    HBVLM::run on the same plan."""
    from oracle import oracle as O
    from tinyvlm_gb300.hbvlm import HBVLM2
    from tinyvlm_gb300.uvlm import kinematics_arrays
    reqs = _requests(seed=9)
    mix, srv = _serve(reqs, lanes=3, concurrent=True)
    # steady
    for r in mix:
        if r.kind != "steady":
            continue
        c = r.payload[0]
        for k, a in enumerate(c.alphas):
            ref = O.vlm_run([c.verts.astype(np.float64)], float(a), dtype=np.float64, ref_pt=(0.25, 0.0, 0.0))
            cl = float(ref["cl"])
            assert abs(r.result[k, 0] - cl) <= 1e-5 * max(abs(cl), 1e-3), (r.rid, r.result[k, 0], cl)
            cm = float(ref["cm"][1])
            assert abs(r.result[k, 3] - cm) <= 1e-5 * max(abs(cm), 1e-3) + 1e-9, (r.rid, r.result[k, 3], cm)
    # UVLM steps: the resident case of _serve (8 x 4 pitch-plunge wing, 10 warm steps)
    steps = [r.result for r in mix if r.kind == "uvlm"]
    uv = S.resident_uvlm(ns=8, nc=4, warm_steps=0, capacity=1)
    last = max(s[0] for s in steps)
    T, Td, fsv, ref = kinematics_arrays(uv.assembly, last + 2, 0.05)
    o = O.uvlm_run([uv.verts], [True], T, Td, fsv, ref, last + 2, 0.05, dtype=np.float32)
    scale = np.abs(o["cl"][1:last + 1]).max()
    for step, cl, _ in steps:
        assert abs(cl - o["cl"][step]) <= 2e-5 * scale, (step, cl, o["cl"][step])
    # HBVLM residuals: the 2-DOF section of hbvlm_factory(nc=10, harmonics=2)
    for r in mix:
        if r.kind != "hbvlm":
            continue
        omega, dyn = r.payload
        hb = HBVLM2("gb300", S.M.rectangular(10, 1, 1.0, 40000.0))
        hb.init(2, 1.0)
        L = hb.plan([hb.parameter_set(omega, dyn)], (0.5,))[0]
        _, out, _ = O.hbvlm_run(hb.verts, [True], 2, omega, L["dt"], L["max_t"], L["wake_T"], L["inst"], L["dft"],
                                L["ddft"], L["force_inst"], L["fs"], L["ref_a"], None, False,
                                np.zeros_like(hb.gamma_coeffs), 1e-9)
        np.testing.assert_allclose(r.result, out[:2], rtol=1e-7, atol=1e-9)
