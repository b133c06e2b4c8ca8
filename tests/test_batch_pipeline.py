"""Host logic of BatchPipeline (several batches in flight): slot turns, first
in first out collection and the refusals, on a stand-in solver that records
its calls (no GPU)."""
import numpy as np
import pytest

from tinyvlm_gb300 import batch as B


class FakeSolver:
    log = []

    def __init__(self, cases, **kw):
        self.id = len([x for x in FakeSolver.log if x[0] == "new"])
        FakeSolver.log.append(("new", self.id))
        self.nsolve, self.gamma_floats, self.tuning = 4, 10, None
        self.inputs = None

    def set_inputs(self, verts, alphas, stream=None, **kw):
        FakeSolver.log.append(("set", self.id, stream))
        self.inputs = np.asarray(alphas).copy()

    def run(self, want_gamma=False, stream=None):
        FakeSolver.log.append(("run", self.id, stream, want_gamma))

    def results_into(self, co, g=None, stream=None):
        FakeSolver.log.append(("read", self.id, stream))
        co[:] = self.inputs[0]
        if g is not None:
            g[:] = self.id

    def launches(self):
        return 7


@pytest.fixture
def fake(monkeypatch):
    FakeSolver.log = []
    monkeypatch.setattr(B, "BatchSolver", FakeSolver)
    return FakeSolver


def test_ring_and_fifo(fake):
    p = B.BatchPipeline([None], depth=3, streams=[11, 12, 13])
    assert [e for e in fake.log if e[0] == "new"] == [("new", 0), ("new", 1), ("new", 2)]
    got = []
    for i in range(8):
        if p.full():
            t, co, _ = p.collect()
            got.append((t, co[0, 0]))
        p.submit(None, [float(i)], want_gamma=(i % 2 == 0))
        assert 1 <= p.pending() <= 3
    while p.pending():
        t, co, _ = p.collect()
        got.append((t, co[0, 0]))
    # every batch comes back once, in submission order, with its own inputs
    assert got == [(i, float(i)) for i in range(8)]
    runs = [(e[1], e[2]) for e in fake.log if e[0] == "run"]
    assert runs == [(i % 3, 11 + i % 3) for i in range(8)]
    # a slot is read back before it takes its next batch
    for i in range(3, 8):
        slot = i % 3
        sets = [k for k, e in enumerate(fake.log) if e[0] == "set" and e[1] == slot]
        reads = [k for k, e in enumerate(fake.log) if e[0] == "read" and e[1] == slot]
        assert all(any(r < s for r in reads) for s in sets[1:])
    assert p.launches() == 7


def test_gamma_only_for_batches_that_stored_it(fake):
    p = B.BatchPipeline([None], depth=2, streams=[1, 2])
    p.submit(None, [1.0], want_gamma=False)
    p.submit(None, [2.0], want_gamma=True)
    with pytest.raises(ValueError, match="without want_gamma"):
        p.collect(g=np.zeros(10, np.float32))
    assert p.pending() == 2  # the refused collect left the batch in flight
    assert p.collect()[0] == 0
    g = np.zeros(10, np.float32)
    t, _, g2 = p.collect(g=g)
    assert t == 1 and g2 is g and (g == 1).all()


def test_refusals(fake):
    with pytest.raises(ValueError, match="at least 1"):
        B.BatchPipeline([None], depth=0, streams=[])
    with pytest.raises(ValueError, match="one stream per slot"):
        B.BatchPipeline([None], depth=2, streams=[1])
    p = B.BatchPipeline([None], depth=1, streams=[5])
    with pytest.raises(RuntimeError, match="no batch in flight"):
        p.collect()
    p.submit(None, [0.0])
    with pytest.raises(RuntimeError, match="collect one first"):
        p.submit(None, [0.0])
    with pytest.raises(RuntimeError, match="in flight first"):
        p.run()
    with pytest.raises(RuntimeError, match="in flight first"):
        p.set_inputs(None, [0.0])
    p.collect()
    p.set_inputs(None, [3.0])
    assert [p.run() for _ in range(3)] == [0, 0, 0]
