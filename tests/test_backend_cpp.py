"""The C++ BackendGB300 (tinyvlm_gb300/backend_cpp) against the reference's
own headers and drivers (CPU: compile and link only).

BackendGB300 subclasses vlm::Backend and creates its Memory, LU, BLAS and
LSQ over libgbvlm.so.  Compiled with g++ against the reference tree's
headers, linked with the reference's vlm/src/*.cpp and its test program
tests/vlm_elliptic_coeffs.cpp, all unmodified, it must build with no
cuBLAS or cuSOLVER.  Run on a host without a GPU, the program stops at the
backend's construction with the reference's print-and-exit convention.
Needs the reference tree (skipped where it is absent, e.g. on the GPU machine).
"""
import glob
import os
import subprocess

import pytest

from oracle.ref import build_ref
from tinyvlm_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.skipif(not build_ref.available(), reason="reference tree not available")


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    build.build()
    ref = build_ref.REF
    out = tmp_path_factory.mktemp("gb300cpp")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "tinyvlm_gb300", "backend_cpp"),
           "-I" + os.path.join(ref, "vlm", "include"), "-I" + os.path.join(ref, "headeronly")]
    cxx = ["g++", "-std=c++17", "-O1", "-w"] + inc
    objs = []
    for src in sorted(glob.glob(os.path.join(ref, "vlm", "src", "*.cpp"))):
        extra = (["-Dcreate_backend=ref_create_backend", "-Dget_available_backends=ref_get_available_backends"]
                 if os.path.basename(src) == "vlm_backend.cpp" else [])
        o = os.path.join(out, os.path.basename(src) + ".o")
        subprocess.run(cxx + extra + ["-c", src, "-o", o], check=True, capture_output=True)
        objs.append(o)
    for src in (os.path.join(ROOT, "tinyvlm_gb300", "backend_cpp", "vlm_backend_gb300.cpp"),
                os.path.join(ROOT, "tests", "cpp", "gb300_factory.cpp")):
        o = os.path.join(out, os.path.basename(src) + ".o")
        r = subprocess.run(cxx + ["-c", src, "-o", o], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        objs.append(o)
    exe = os.path.join(out, "vlm_elliptic_coeffs_gb300")
    libdir = os.path.dirname(build.LIB)
    r = subprocess.run(cxx + [os.path.join(ref, "tests", "vlm_elliptic_coeffs.cpp")] + objs +
                       ["-L" + libdir, "-lgbvlm", "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_links_without_vendor_libraries(program):
    r = subprocess.run(["ldd", program], capture_output=True, text=True)
    assert "libgbvlm.so" in r.stdout
    for vendor in ("libcublas", "libcusolver"):
        assert vendor not in r.stdout


def test_reference_driver_stops_cleanly_without_a_gpu(program):
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    run = os.path.join(build_ref.OUT, "run", "a", "b", "c", "d")
    os.makedirs(run, exist_ok=True)
    r = subprocess.run([program], capture_output=True, text=True, cwd=run, timeout=120)
    assert r.returncode == 1, (r.returncode, r.stdout[-500:], r.stderr[-500:])
    assert "gbvlm error in" in r.stderr
