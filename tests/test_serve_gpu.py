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
