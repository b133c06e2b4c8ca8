"""The C-ABI library builds, loads and exports every entry point that
include/gbvlm.h declares (no compute calls: runs without a GPU)."""
import os
import re

from tinyvlm_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gbvlm.h")


def declared():
    with open(HEADER) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbvlm_[a-z0-9_]+)\s*\(", src)))


def test_header_parses():
    names = declared()
    assert "gbvlm_lhs_assemble_f32" in names and "gbvlm_lu_factor_f64" in names
    assert len(names) > 40


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing


def test_python_prototypes_cover_header():
    names = set(declared())
    assert names <= set(_lib.exported_names()) | {"gbvlm_last_error", "gbvlm_version"}, \
        names - set(_lib.exported_names())


def test_library_is_in_tree():
    assert os.path.dirname(build.LIB) == os.path.dirname(os.path.abspath(_lib.__file__))


def test_argument_checks_need_no_gpu():
    """Entry points validate their arguments before touching the device and
    report GBVLM_ERR_ARG (1) with a message; nothing aborts the process."""
    L = _lib.lib()
    P = None
    cases = [
        ("gbvlm_hbvlm_prepare_batch", (P, 2, 2, P, P, P, P, P, P, P, P), b"null argument"),
        ("gbvlm_hbvlm_prepare_batch_chain", (P, 2, 2, P, P, P, P, P, P, P, P), b"null argument"),
        ("gbvlm_hbvlm_solve_batch", (P, 2, P, P, P, 100, 1e-9, 10, P, P), b"solve before prepare"),
        ("gbvlm_hbvlm_loads_batch", (P, 2, P, P, P, P, P, P, P, P, 0, P, P), b"null argument"),
        ("gbvlm_test_flow_wait_timeout", (64, P), b"n must span"),
    ]
    for name, args, msg in cases:
        rc = getattr(L, name)(*args)
        assert rc == 1, (name, rc)
        assert msg in L.gbvlm_last_error(), (name, L.gbvlm_last_error())
