"""The autotuner's keys and table lookup are deterministic (CPU: the tuning
table of the library is host state; no kernel runs)."""
import json
import os

import numpy as np
import pytest

from tinyvlm_gb300 import autotune as A
from tinyvlm_gb300 import mesh as M


@pytest.fixture(autouse=True)
def _restore():
    yield
    A.reset()


def test_parameters_and_defaults():
    p = A.params()
    assert set(p) >= {"wake.waves", "hbvlm.waves", "hbvlm.min_rows", "batch.group_hi", "batch.group_lo",
                      "batch.loads_threads", "batch.assembly_span", "batch.assembly_rows", "batch.group_mid"}
    d = A.defaults()
    assert d["wake.waves"] == 4 and d["batch.group_hi"] == 1024 and d["batch.group_lo"] == 384
    assert d["batch.assembly_span"] == 128 and d["batch.loads_threads"] == 0 and d["batch.assembly_rows"] == 4
    assert d["batch.group_mid"] == 0
    with pytest.raises(Exception):
        A.set_params({"batch.assembly_span": 96})
    with pytest.raises(Exception):
        A.set_params({"batch.assembly_rows": 5})
    with pytest.raises(Exception):
        A.set_params({"no.such": 1})
    assert A.current() == d


def test_keys_are_deterministic_and_order_free():
    cases = M.batch_cases(64, seed=3, n_alpha=8)
    dims = [(c.ns, c.nc) for c in cases]
    na = [len(c.alphas) for c in cases]
    k1 = A.batch_key(dims, na, "shared", 1, 152)
    assert k1 == A.batch_key(list(reversed(dims)), list(reversed(na)), "shared", 1, 152)
    assert k1 != A.batch_key(dims, na, "exact", 1, 152) and k1 != A.batch_key(dims, na, "shared", 1, 148)
    assert A.wake_key(1600, 20000, 152) == A.wake_key(1600, 20000, 152)
    assert A.wake_key(1600, 16384, 152) == A.wake_key(1600, 17000, 152)  # same power-of-two bucket


def test_lookup_is_deterministic_and_table_entries_are_valid():
    t = A.table()
    assert t["version"] == 1
    ranges = A.params()
    for key, e in t["entries"].items():
        first = A.lookup(key)
        assert first == A.lookup(key) == e["params"]
        for name, v in e["params"].items():
            lo, hi = ranges[name]
            assert lo <= v <= hi, (key, name, v)
        applied = A.apply(key)
        assert applied["source"] == "table" and applied["params"] == {
            **{k: v for k, v in A.defaults().items() if k.startswith(key.split("/")[0] + ".")}, **first}
        for name, v in first.items():
            assert A.get(name) == v
        A.reset()
    missing = A.apply("batch/shared/r1/sm1/c1/p1/m1/a1")
    assert missing["source"] == "default" and A.current() == A.defaults()


def test_headline_workload_has_a_tuned_entry():
    """The benchmark's batched workload (512 seeded trapezoids x 8 alphas) on a 152-SM GB300."""
    cases = M.batch_cases(512, seed=20261203, n_alpha=8)
    key = A.batch_key([(c.ns, c.nc) for c in cases], [8] * 512, "shared", 1, 152)
    if not os.path.exists(A.TABLE):
        pytest.skip("no tuning table yet")
    assert A.lookup(key) is not None, key


def test_batch_key_in_flight():
    """Batches in flight enter the key only when more than one, so one-in-flight keys stay as they were."""
    dims, na = [(8, 4), (16, 8)], [8, 8]
    k1 = A.batch_key(dims, na, "shared", 1, 152)
    assert A.batch_key(dims, na, "shared", 1, 152, in_flight=1) == k1
    assert A.batch_key(dims, na, "shared", 1, 152, in_flight=2) == k1 + "/f2"
