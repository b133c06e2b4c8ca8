"""ctypes binding of libgbvlm.so (the C ABI declared in include/gbvlm.h).

The library is built in-tree by ``tinyvlm_gb300.build``.  There is no CPU
fallback: if the shared library is missing or cannot be loaded, every entry
point raises.
"""
import ctypes
import os

from . import build as _build

P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
F32 = ctypes.c_float
F64 = ctypes.c_double
PP = ctypes.POINTER(ctypes.c_void_p)


class Dims(ctypes.Structure):
    _fields_ = [("ns", I64), ("nc", I64), ("nwv", I64)]


class Coeffs(ctypes.Structure):
    _fields_ = [("cl", F64), ("cdi", F64), ("cm", F64 * 3)]


GBVLM_OK = 0
ERRORS = {1: "GBVLM_ERR_ARG", 2: "GBVLM_ERR_CUDA", 3: "GBVLM_ERR_SINGULAR", 4: "GBVLM_ERR_NOMEM",
          5: "GBVLM_ERR_IO", 6: "GBVLM_ERR_STATE"}
ERRORS_BY_NAME = {v: k for k, v in ERRORS.items()}


class GbvlmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, str(code)), msg))
        self.code = code


def _protos():
    t = {}
    for sfx, R in (("f32", F32), ("f64", F64)):
        t["gbvlm_lhs_assemble_" + sfx] = [P, I64, I32, P, PP, PP, PP, PP, I32, R, P]
        t["gbvlm_rhs_assemble_velocities_" + sfx] = [P, I32, P, PP, PP, P]
        t["gbvlm_rhs_assemble_wake_influence_" + sfx] = [P, I32, P, PP, PP, PP, PP, P, I32, R, P]
        t["gbvlm_forces_steady_" + sfx] = [I64, I64, P, P, P, P, P]
        t["gbvlm_forces_unsteady_" + sfx] = [I64, I64, P, P, P, P, P, P, P, P]
        t["gbvlm_coeff_cl_" + sfx] = [I64, I64, P, P, P, R, R, P, P]
        t["gbvlm_coeff_cm_" + sfx] = [I64, I64, P, P, P, P, R, R, R, P, P]
        t["gbvlm_mesh_metrics_" + sfx] = [R, I32, P, PP, PP, PP, PP, P]
        t["gbvlm_mesh_mac_" + sfx] = [I64, I64, P, P, P, P]
        t["gbvlm_gamma_wake_from_coeffs_" + sfx] = [P, I64, I64, P, I32, R, R, R, I64, P]
        t["gbvlm_sum_" + sfx] = [P, I64, P, P]
        t["gbvlm_displace_wing_" + sfx] = [I32, P, PP, PP, PP, P]
        t["gbvlm_wake_shed_" + sfx] = [I32, P, PP, PP, I32, P]
        t["gbvlm_wake_rollup_" + sfx] = [I32, P, PP, PP, PP, PP, P, R, R, I32, P]
        t["gbvlm_trefftz_cd_" + sfx] = [I64, I64, P, P, P, R, R, P, P]
        t["gbvlm_gamma_update_" + sfx] = [I64, I64, P, P, P, P, I64, P, P, R, P]
        t["gbvlm_lu_factor_" + sfx] = [P, P, I64, I64, P]
        t["gbvlm_lu_solve_" + sfx] = [P, P, I64, I64, P, I64, I64, P]
        t["gbvlm_sum2d_" + sfx] = [P, I64, I64, I64, I64, P, P]
        t["gbvlm_mem_fill_" + sfx] = [I32, P, I64, R, I64, P]
        t["gbvlm_blas_gemv_" + sfx] = [I32, I64, I64, R, P, I64, P, I64, R, P, I64, P]
        t["gbvlm_blas_gemm_" + sfx] = [I32, I32, I64, I64, I64, R, P, I64, P, I64, R, P, I64, P]
        t["gbvlm_blas_axpy_" + sfx] = [I64, R, P, I64, P, I64, P]
        t["gbvlm_blas_axpy2d_" + sfx] = [I64, I64, R, P, I64, I64, P, I64, I64, P]
        t["gbvlm_blas_scal_" + sfx] = [I64, R, P, I64, P]
        t["gbvlm_blas_nrm2_" + sfx] = [I64, P, I64, P, P]
        t["gbvlm_lsq_solve_" + sfx] = [I64, I64, P, I64, P, I64, I64, P]
    t["gbvlm_tune_set"] = [ctypes.c_char_p, I64]
    t["gbvlm_tune_get"] = [ctypes.c_char_p, P]
    t["gbvlm_tune_reset"] = []
    t["gbvlm_tune_count"] = [P]
    t["gbvlm_tune_name"] = [I32, P, P, P]
    t["gbvlm_mem_alloc"] = [I32, I64, P]
    t["gbvlm_mem_free"] = [I32, P]
    t["gbvlm_mem_copy"] = [I32, P, I64, I32, P, I64, I64, I64, P]
    t["gbvlm_stream_create"] = [P]
    t["gbvlm_stream_destroy"] = [P]
    t["gbvlm_stream_synchronize"] = [P]
    t["gbvlm_device_synchronize"] = []
    t["gbvlm_event_create"] = [P]
    t["gbvlm_event_destroy"] = [P]
    t["gbvlm_event_record"] = [P, P]
    t["gbvlm_event_synchronize"] = [P]
    t["gbvlm_event_elapsed_ms"] = [P, P, P]
    t["gbvlm_device_info"] = [P, P, P]
    t["gbvlm_rhs_assemble_wake_influence_f32_noalloc"] = [P, I32, P, PP, PP, PP, PP, P, I32, F32, P]
    t["gbvlm_lu_create"] = [P]
    t["gbvlm_lu_destroy"] = [P]
    t["gbvlm_lu_init"] = [P, I64]
    t["gbvlm_lu_solve_refined"] = [P, P, P, I64, I64, P, P, I64, I32, P, P]
    t["gbvlm_vlm_create"] = [P, I32, P, PP, I32]
    t["gbvlm_vlm_destroy"] = [P]
    t["gbvlm_vlm_run"] = [P, F64, F64, F64, F64, P, P, P, P]
    t["gbvlm_vlm_run_shared"] = [P, I32, P, F64, F64, P, P, P, P]
    t["gbvlm_read_plot3d"] = [ctypes.c_char_p, I32, P, P]
    t["gbvlm_test_flow_wait_timeout"] = [I32, P]
    t["gbvlm_test_tc_wait_timeout"] = [P]
    t["gbvlm_nlvlm_create"] = [P, I32, P, PP, I32]
    t["gbvlm_nlvlm_destroy"] = [P]
    t["gbvlm_nlvlm_run"] = [P, F64, F64, F64, F64, P, P, I32, F64, I32, P, P, P, P, P]
    t["gbvlm_batch_create"] = [P, I32, P, P, I32, I32]
    t["gbvlm_batch_create_ex"] = [P, I32, P, P, I32, I32, I32]
    t["gbvlm_batch_destroy"] = [P]
    t["gbvlm_batch_info"] = [P, P, P, P, P, P, P]
    t["gbvlm_batch_set_inputs"] = [P, P, P, F64, F64, P, P]
    t["gbvlm_batch_run"] = [P, I32, P]
    t["gbvlm_batch_run_eager"] = [P, I32, P]
    t["gbvlm_batch_results"] = [P, P, P, P]
    t["gbvlm_batch_profile"] = [P, P, P]
    t["gbvlm_batch_update_profile"] = [P, P, P]
    t["gbvlm_batch_launches"] = [P, P]
    t["gbvlm_uvlm_create"] = [P, I32, P, PP, P, I64, I32]
    t["gbvlm_uvlm_destroy"] = [P]
    t["gbvlm_uvlm_set_kinematics"] = [P, P, P, P, P]
    t["gbvlm_uvlm_run"] = [P, F64, I32, F64, P]
    t["gbvlm_uvlm_results"] = [P, P, P, P, P]
    t["gbvlm_uvlm_begin"] = [P, F64, I32, F64, P]
    t["gbvlm_uvlm_step"] = [P, P, P, P, P]
    t["gbvlm_uvlm_step_graph"] = [P, P, P, P, P]
    t["gbvlm_uvlm_loop_create"] = [P, P, F64]
    t["gbvlm_uvlm_loop_submit"] = [P, P]
    t["gbvlm_uvlm_loop_wait"] = [P, I64, F64, P, P, P]
    t["gbvlm_uvlm_loop_stats"] = [P, P, P, P]
    t["gbvlm_uvlm_loop_destroy"] = [P]
    t["gbvlm_newmark_create"] = [P, F64, F64]
    t["gbvlm_newmark_destroy"] = [P]
    t["gbvlm_newmark_init"] = [P, I32, P, P, P, F64, P]
    t["gbvlm_newmark_step"] = [P, P, P, P, P, P, P, P, P, F64, P]
    t["gbvlm_aero2dof_create"] = [P, I32, P, PP, P, P, F64, P, P, P]
    t["gbvlm_aero2dof_destroy"] = [P]
    t["gbvlm_aero2dof_run"] = [P, I64, I32, P]
    t["gbvlm_aero2dof_results"] = [P, P, P, P, P, P, P, P]
    t["gbvlm_hbvlm_create"] = [P, I32, P, PP, P]
    t["gbvlm_hbvlm_destroy"] = [P]
    t["gbvlm_hbvlm_prepare"] = [P, I32, I64, P, P, P, P, P, P, P]
    t["gbvlm_hbvlm_map"] = [P, P, P, F64, F64, P]
    t["gbvlm_hbvlm_solve"] = [P, P, F64, F64, I32, F64, I32, P, P]
    t["gbvlm_hbvlm_loads"] = [P, P, P, P, P, P, P, P, P, I32, P, P]
    t["gbvlm_hbvlm_prepare_batch"] = [P, I32, I32, P, PP, P, P, P, P, P, P]
    t["gbvlm_hbvlm_prepare_batch_chain"] = [P, I32, I32, P, P, P, P, P, P, P, P]
    t["gbvlm_hbvlm_solve_batch"] = [P, I32, P, P, P, I32, F64, I32, P, P]
    t["gbvlm_hbvlm_loads_batch"] = [P, I32, P, P, P, P, P, P, P, P, I32, P, P]
    return t


_LIB = None


def lib():
    """Load (building first if needed) and return the ctypes library."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if not os.path.exists(path) or _build.stale():
            _build.build()
        L = ctypes.CDLL(path)
        L.gbvlm_last_error.restype = ctypes.c_char_p
        L.gbvlm_version.restype = ctypes.c_int
        for name, args in _protos().items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _LIB = L
    return _LIB


def exported_names():
    return sorted(_protos().keys()) + ["gbvlm_last_error", "gbvlm_version"]


def call(name, *args):
    L = lib()
    rc = getattr(L, name)(*args)
    if rc != GBVLM_OK:
        raise GbvlmError(rc, L.gbvlm_last_error().decode(errors="replace"))
    return rc


def ptr_array(ptrs):
    arr = (ctypes.c_void_p * len(ptrs))(*[ctypes.c_void_p(p) for p in ptrs])
    return ctypes.cast(arr, PP), arr


def dims_array(dims):
    arr = (Dims * len(dims))(*[Dims(int(a), int(b), int(c)) for a, b, c in dims])
    return arr
