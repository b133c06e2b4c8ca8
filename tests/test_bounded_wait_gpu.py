"""Failure path of the bounded waits: the dataflow triangular solve's wait
for a block that never finishes, and a tensor-core update tile's wait for
MMAs that are never committed, run out (2 s); the launch reports it as an
error with its message, and the CUDA context stays usable (a batch solve
afterwards gives the right answer).  No fault, trap or hang: the waits are
polled (a counter, an mbarrier) with a time limit, and the withheld work is
work that is never issued."""
import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import _lib
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts

pytestmark = pytest.mark.gpu


def test_wait_runs_out_and_context_survives(cuda):
    L = _lib.lib()
    rc = L.gbvlm_test_flow_wait_timeout(256, None)
    assert rc == 2, rc  # GBVLM_ERR_CUDA
    assert b"timed out" in L.gbvlm_last_error()
    cases = M.batch_cases(3, seed=4, n_alpha=2, nc_range=(4, 8), ns_range=(8, 16))
    bs = BatchSolver(cases, mode="shared", refine=1)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=(0.25, 0.0, 0.0))
    bs.run()
    co, _ = bs.results()
    k = 0
    for c in cases:
        for r in O.vlm_shared([c.verts.astype(np.float64)], c.alphas, ref_pt=(0.25, 0.0, 0.0)):
            assert abs(co[k, 0] - float(r["cl"])) <= 1e-5 * max(abs(float(r["cl"])), 1e-3)
            k += 1


def test_tensor_core_tile_wait_runs_out_and_context_survives(cuda):
    L = _lib.lib()
    rc = L.gbvlm_test_tc_wait_timeout(None)
    assert rc == 2, (rc, L.gbvlm_last_error())  # GBVLM_ERR_CUDA
    assert b"timed out" in L.gbvlm_last_error()
    test_wait_runs_out_and_context_survives(cuda)
