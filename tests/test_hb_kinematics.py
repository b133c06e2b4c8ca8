"""The closed-form kinematics of the HBVLM modules against the kinematics
tree (Dual evaluation of the chain the modules build, libhbvlm3.cpp:559-641
and libhbvlm.cpp:470-515), for several parameter sets."""
import numpy as np

from tinyvlm_gb300 import hbvlm as HB


def _sets(rng, K, H, nd, with_U):
    sets = []
    for _ in range(K):
        d = rng.uniform(-0.05, 0.05, (nd, 2 * H + 1))
        S = dict(omega=float(rng.uniform(0.3, 1.2)), dyn=d)
        if with_U:
            S["U"] = float(rng.uniform(5.0, 12.0))
        sets.append(S)
    return sets


def _check(obj, sets, tree_nodes):
    rng = np.random.default_rng(1)
    times = [np.sort(rng.uniform(0.0, 40.0, 37 + 5 * k)) for k in range(len(sets))]
    worst = 0.0
    for k, S in enumerate(sets):
        series = obj._series(S, times[k])
        sl = slice(0, times[k].size)
        for m, node in enumerate(tree_nodes(S)):
            v, g = node.transform_series(times[k])
            worst = max(worst, np.abs(series[m][0][sl] - v).max(), np.abs(series[m][1][sl] - g).max())
            np.testing.assert_allclose(series[m][0][sl], v, rtol=0, atol=1e-14)
            np.testing.assert_allclose(series[m][1][sl], g, rtol=0, atol=1e-13)
    return worst


def test_hbvlm2_chain():
    obj = HB.HBVLM2.__new__(HB.HBVLM2)
    obj.m_harmonics = 3
    sets = _sets(np.random.default_rng(0), 4, 3, 2, False)
    w = _check(obj, sets, lambda S: obj.assembly(S["omega"], S["dyn"]).surface_kinematics())
    print("max difference", w)


def test_hbvlm3_chain_wing_and_flap():
    obj = HB.HBVLM3.__new__(HB.HBVLM3)
    obj.m_harmonics = 2
    sets = _sets(np.random.default_rng(2), 3, 2, 3, True)
    w = _check(obj, sets, lambda S: obj.assembly(S["omega"], S["U"], S["dyn"]).surface_kinematics())
    print("max difference", w)
    # the free stream rate the loads use
    S = sets[0]
    _, da = obj.assembly(S["omega"], S["U"], S["dyn"]).kinematics().transform_series(np.array([0.0, 1.0]))
    np.testing.assert_array_equal(-da[:, 0, 3], obj._sigma(S))


def test_sets_evaluated_together_equal_one_at_a_time():
    """The batch path evaluates the instances of all parameter sets in one
    vectorised pass (per-element omega, speed and coefficient rows): each
    set's transforms equal its own evaluation bitwise."""
    for cls, nd, with_U, H in ((HB.HBVLM2, 2, False, 3), (HB.HBVLM3, 3, True, 2)):
        obj = cls.__new__(cls)
        obj.m_harmonics = H
        sets = _sets(np.random.default_rng(4), 5, H, nd, with_U)
        rng = np.random.default_rng(6)
        times = [np.sort(rng.uniform(0.0, 30.0, 7)) for _ in sets]
        own = np.concatenate([np.full(t.size, k) for k, t in enumerate(times)])
        together = obj._chain_series(sets, own, np.concatenate(times))
        off = 0
        for S, t in zip(sets, times):
            alone = obj._series(S, t)
            for m in range(len(alone)):
                np.testing.assert_array_equal(together[m][0][off:off + t.size], alone[m][0])
                np.testing.assert_array_equal(together[m][1][off:off + t.size], alone[m][1])
            off += t.size


def test_chain_vector_layout():
    """k_hb_chain's parameters: sigma, omega, dt, px, qx, flap, then the heave, pitch and control rows."""
    obj = HB.HBVLM3.__new__(HB.HBVLM3)
    obj.m_harmonics, obj.m_coeffs = 2, 5
    S = dict(omega=0.9, U=8.0, dyn=np.arange(15.0).reshape(3, 5))
    v = obj._chain_vector(S, 0.01)
    assert v.shape == (6 + 3 * 5,)
    # the free stream speed uses the reference's float-literal constants (libhbvlm3.cpp:562-581)
    b, w_a = float(np.float32(0.127)), float(np.float32(52.6506))
    np.testing.assert_array_equal(v[:6], [8.0 / (b * w_a), 0.9, 0.01, 0.5, 1.5, 1.0])
    np.testing.assert_array_equal(v[6:], np.arange(15.0))
    obj2 = HB.HBVLM2.__new__(HB.HBVLM2)
    obj2.m_harmonics, obj2.m_coeffs = 2, 5
    v2 = obj2._chain_vector(dict(omega=0.4, dyn=np.ones((2, 5))), 0.02)
    np.testing.assert_array_equal(v2[:6], [1.0, 0.4, 0.02, 0.5, 0.0, 0.0])
    np.testing.assert_array_equal(v2[16:], np.zeros(5))
