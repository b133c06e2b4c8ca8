"""Accuracy of the headline batched workload as the benchmark runs it: 512
trapezoidal wings (seed 20261203) x 8 alpha on the shared-AIC formulation,
float assembly and 3xTF32 tensor-core LU, one refinement sweep with a
double residual (the benchmark's default).  Without the sweep the worst of
the 4096 solves sits near 1.4e-5 (the fp32 factorisation's floor).  Every one of the
4096 solves against the double oracle (double geometry, assembly and LAPACK
dgetrf/dgetrs): CL and CM within a relative 1e-5 (CL relative to
max(|CL|, 1e-3 max|CL|) so that alpha near zero is not divided by ~0)."""
import numpy as np
import pytest

from oracle import oracle as O
from tinyvlm_gb300 import mesh as M
from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts

pytestmark = pytest.mark.gpu
REF = (0.25, 0.0, 0.0)


def test_headline_batch_cl_cm_within_1e5(cuda):
    cases = M.batch_cases(512, seed=20261203, n_alpha=8)
    bs = BatchSolver(cases, mode="shared", refine=1)
    bs.set_inputs(pack_verts(cases), pack_alphas(cases), ref_pt=REF)
    bs.run()
    co, _ = bs.results()
    cl_ref, cm_ref = [], []
    for c in cases:
        for r in O.vlm_shared([c.verts.astype(np.float64)], c.alphas, ref_pt=REF):
            cl_ref.append(float(r["cl"]))
            cm_ref.append(np.asarray(r["cm"], np.float64))
    cl_ref = np.array(cl_ref)
    cm_ref = np.array(cm_ref)
    guard = 1e-3 * np.abs(cl_ref).max()
    cl_err = np.abs(co[:, 0] - cl_ref) / np.maximum(np.abs(cl_ref), guard)
    cm_scale = np.maximum(np.abs(cm_ref).max(axis=1), 1e-6)
    cm_err = np.abs(co[:, 2:5] - cm_ref).max(axis=1) / cm_scale
    print("headline batch: max rel err CL %.3e, CM %.3e over %d solves" % (cl_err.max(), cm_err.max(), len(cl_err)))
    assert cl_err.max() <= 1e-5, (int(cl_err.argmax()), cl_err.max())
    assert cm_err.max() <= 1e-5, (int(cm_err.argmax()), cm_err.max())
