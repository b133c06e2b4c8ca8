"""Recipe for oracle/_ref: the reference's own driver code, compiled here.

Test infrastructure only.  It compiles, unmodified and in place, the
reference's simulation drivers (vlm/src/*.cpp), its CPU backend host code
(vlm/backends/cpu/src/*.cpp), its harmonic-balance module (lib/libhbvlm3.cpp)
and its test programs (tests/*.cpp), and links them against:

  * oracle/ref/ispc_kernels.c + oracle/vlm_oracle.c: the four ISPC kernels
    (no ispc compiler here), restated in plain C;
  * oracle/ref/include/taskflow/: a stand-in for the Taskflow calls of the
    backend (the library is fetched from the network by the reference's
    build);
  * oracle/ref/include/{lapacke,cblas}.h: LAPACKE/CBLAS prototypes bound to
    scipy's bundled OpenBLAS.

Nothing from the reference is copied: every reference file is read from the
reference tree (TINYVLM_REF, default /root/reference) by the compiler.
Outputs go to oracle/_ref/ only (git-ignored):

  libvlm_ref.so             drivers + CPU backend + kernels
  ref_fixtures              oracle/ref/ref_fixtures.cpp (our driver program)
  vlm_elliptic_coeffs ...   the reference's test programs
  libhbvlm3.<ext>           the reference's pybind module

Run:  python -m oracle.ref.build_ref [--force]
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
OBJ = os.path.join(OUT, "obj")
REF = os.environ.get("TINYVLM_REF", "/root/reference")

TESTS = ["vlm_elliptic_coeffs", "vlm_square_coeffs", "uvlm_theodorsen", "nlvlm_curves", "ut_kinematics",
         "ut_tensor", "newmark"]


def available():
    return os.path.isdir(os.path.join(REF, "vlm", "src"))


def _openblas():
    import scipy
    libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cands = [p for p in glob.glob(os.path.join(libs, "libscipy_openblas*.so")) if "64_" not in os.path.basename(p)]
    if not cands:
        raise RuntimeError("scipy's bundled OpenBLAS not found under " + libs)
    return libs, os.path.basename(cands[0])


def _includes():
    return ["-I" + os.path.join(HERE, "include"), "-I" + os.path.join(REF, "vlm", "include"),
            "-I" + os.path.join(REF, "vlm", "backends", "cpu", "include"), "-I" + os.path.join(REF, "headeronly")]


CXX = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-DVLM_CPU", "-w"]
CC = ["gcc", "-std=c11", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("failed: %s\n%s" % (" ".join(cmd), r.stderr[-4000:]))


def _obj(src):
    return os.path.join(OBJ, os.path.basename(src) + ".o")


def build(force=False):
    if not available():
        raise RuntimeError("reference tree not found at %s (set TINYVLM_REF)" % REF)
    lib = os.path.join(OUT, "libvlm_ref.so")
    if not force and os.path.exists(lib) and os.path.exists(os.path.join(OUT, "ref_fixtures")):
        return OUT
    os.makedirs(OBJ, exist_ok=True)
    libdir, blas = _openblas()
    cxx_srcs = sorted(glob.glob(os.path.join(REF, "vlm", "src", "*.cpp"))) + \
        sorted(glob.glob(os.path.join(REF, "vlm", "backends", "cpu", "src", "*.cpp")))
    jobs = [CXX + _includes() + ["-c", s, "-o", _obj(s)] for s in cxx_srcs]
    jobs += [CC + ["-c", os.path.join(ORACLE, "vlm_oracle.c"), "-o", _obj("vlm_oracle.c")],
             CC + ["-I" + os.path.join(HERE, "include"), "-c", os.path.join(HERE, "ispc_kernels.c"),
                   "-o", _obj("ispc_kernels.c")]]
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    objs = [_obj(s) for s in cxx_srcs] + [_obj("vlm_oracle.c"), _obj("ispc_kernels.c")]
    link = ["-L" + libdir, "-l:" + blas, "-Wl,-rpath," + libdir, "-lm"]
    _run(CXX + ["-shared", "-o", lib] + objs + link)
    use = ["-L" + OUT, "-lvlm_ref", "-Wl,-rpath,$ORIGIN"] + link
    progs = [(os.path.join(HERE, "ref_fixtures.cpp"), "ref_fixtures")]
    progs += [(os.path.join(REF, "tests", t + ".cpp"), t) for t in TESTS]
    jobs = [CXX + _includes() + [src, "-o", os.path.join(OUT, name)] + use for src, name in progs]
    import pybind11
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    pyinc = sysconfig.get_paths()["include"]
    jobs.append(CXX + _includes() + ["-I" + pyinc, "-I" + pybind11.get_include(), "-shared",
                                     os.path.join(REF, "lib", "libhbvlm3.cpp"),
                                     "-o", os.path.join(OUT, "libhbvlm3" + ext)] + use)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    # the reference's tests open meshes at ../../../../mesh/<name>: run them
    # from run/a/b/c/d with run/mesh pointing at the reference's meshes
    run = os.path.join(OUT, "run")
    os.makedirs(os.path.join(run, "a", "b", "c", "d"), exist_ok=True)
    link_mesh = os.path.join(run, "mesh")
    if not os.path.islink(link_mesh):
        os.symlink(os.path.join(REF, "mesh"), link_mesh)
    return OUT


def test_cwd():
    """Working directory from which the reference's test programs find their meshes."""
    return os.path.join(OUT, "run", "a", "b", "c", "d")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
