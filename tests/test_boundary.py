"""Boundary checks that need no GPU: the Python layer imports without
PyTorch, and the library's C plot3d reader (gbvlm_read_plot3d, a host
routine) reproduces the reference reader (vlm/src/vlm_mesh.cpp:16-92) on
the reference's meshes, quarter-chord shift included, bit for bit."""
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from tests import ref_fixtures as R
from tinyvlm_gb300 import mesh as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_package_imports_without_pytorch():
    code = r'''
import sys, importlib.abc
class Block(importlib.abc.MetaPathFinder):
    def find_spec(self, name, path, target=None):
        if name == "torch" or name.startswith("torch."):
            raise ImportError("torch is blocked")
        return None
sys.meta_path.insert(0, Block())
import tinyvlm_gb300
from tinyvlm_gb300 import backend, batch, device, hbvlm, integrator, kinematics, mesh, serve, uvlm, vlm, aeroelastic
from tinyvlm_gb300 import finite_diff
from tinyvlm_gb300.compat import libhbvlm, libhbvlm3
assert "torch" not in sys.modules
print("ok")
'''
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stderr[-2000:]


@pytest.mark.parametrize("name", ["elliptic_16x16", "elliptic_45x45", "swept_4x4", "infinite_rectangular_2x2_part0",
                                  "infinite_rectangular_5x200", "3dof_flap_15x1"])
def test_c_plot3d_reader_matches_reference_reader(name):
    from tinyvlm_gb300.vlm import read_plot3d
    raw = R.raw_mesh(name)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, name + ".x")
        M.write_plot3d(p, raw)
        assert np.array_equal(read_plot3d(p, qc=False), raw)
        assert np.array_equal(read_plot3d(p), R.mesh(name))


def test_c_plot3d_reader_rejects_what_the_reference_rejects():
    from tinyvlm_gb300._lib import GbvlmError
    from tinyvlm_gb300.vlm import read_plot3d
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "two_blocks.x")
        with open(p, "w") as f:
            f.write("2\n3 3 1\n")
        with pytest.raises(GbvlmError):
            read_plot3d(p)
        p = os.path.join(d, "spanwise_rows.x")  # first spanwise row with varying y (vlm_mesh.cpp:84-91)
        v = M.rectangular(2, 3, 1.0, 3.0)
        M.write_plot3d(p, v.transpose(0, 2, 1))
        with pytest.raises(GbvlmError):
            read_plot3d(p)
        with pytest.raises(GbvlmError):
            read_plot3d(os.path.join(d, "missing.x"))
