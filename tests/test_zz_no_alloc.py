"""The allocation-free wake-influence entry point gives the same right-hand
side as the regular one, bit for bit.

It exists for callers that cannot allocate device memory: a host
application whose device memory belongs to its own allocator, a serving
loop held to a fixed device-memory budget, a latency path that must not
take cudaMalloc's device-wide synchronisation.  Its partial sums live in a
fixed array inside the library.  Both entry points run the same kernels
with the same slice count, so the results must be identical.  Two calls in
a row with different wakes check that nothing from the first call leaks
into the second.  This file sorts last so a failure here stops a `-x` run
only after every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from tests.helpers import synthetic_wake, wing
from tinyvlm_gb300 import _lib
from tinyvlm_gb300._lib import F32, call, dims_array, ptr_array

pytestmark = pytest.mark.gpu


def _inputs(seed, rows, iteration):
    from oracle import oracle as O
    surf = [wing("rect", 5, 12), wing("trap", 4, 9)]
    col, nor, _ = O.mesh_metrics(0.0, surf, np.float32)
    wakes = [synthetic_wake(s, rows, seed=seed + i) for i, s in enumerate(surf)]
    rng = np.random.default_rng(seed)
    gw = [rng.standard_normal((rows - 1, s.shape[2] - 1)).astype(np.float32) for s in surf]
    dims = dims_array([(s.shape[2] - 1, s.shape[1] - 1, rows) for s in surf])
    dev = lambda xs: [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in xs]
    return dims, dev(gw), dev(col), dev(nor), dev(wakes), iteration


def _call(name, rhs, dims, gw, col, nor, wakes, iteration):
    keep = []
    arrs = []
    for group in (gw, col, nor, wakes):
        a, k = ptr_array([t.data_ptr() for t in group])
        arrs.append(a)
        keep.append(k)
    lf = (ctypes.c_int32 * 2)(1, 1)
    call(name, ctypes.c_void_p(rhs.data_ptr()), 2, dims, *arrs, ctypes.cast(lf, ctypes.c_void_p), int(iteration),
         F32(0.0), None)


@pytest.mark.parametrize("first,second", [((1, 30, 29), (2, 40, 17))])
def test_noalloc_matches_regular_entry_point(cuda, first, second):
    for seed, rows, it in (first, second):
        dims, gw, col, nor, wakes, it = _inputs(seed, rows, it)
        n = sum(int(c.shape[1] * c.shape[2]) for c in col)
        base = torch.linspace(-1.0, 1.0, n, device="cuda", dtype=torch.float32)
        want = base.clone()
        got = base.clone()
        _call("gbvlm_rhs_assemble_wake_influence_f32", want, dims, gw, col, nor, wakes, it)
        _call("gbvlm_rhs_assemble_wake_influence_f32_noalloc", got, dims, gw, col, nor, wakes, it)
        torch.cuda.synchronize()
        g, w = got.cpu().numpy(), want.cpu().numpy()
        assert not np.array_equal(w, base.cpu().numpy()), "the wake added nothing"
        assert np.array_equal(g, w), "no-alloc wake rhs differs: max |diff| %g" % np.abs(g - w).max()


def test_noalloc_rejects_too_many_points(cuda):
    dims = dims_array([(2048, 1024, 3)])
    z = torch.zeros(4, device="cuda")
    a, k = ptr_array([z.data_ptr()])
    lf = (ctypes.c_int32 * 1)(1)
    with pytest.raises(_lib.GbvlmError, match="fixed scratch"):
        call("gbvlm_rhs_assemble_wake_influence_f32_noalloc", ctypes.c_void_p(z.data_ptr()), 1, dims, a, a, a, a,
             ctypes.cast(lf, ctypes.c_void_p), 1, F32(0.0), None)
