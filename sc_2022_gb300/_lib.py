"""ctypes binding of libsbpmg.so (the C ABI declared in include/sbpmg.h).

The library is loaded from this package directory.  There is no fallback:
if the shared library is missing the import fails with instructions to run
the build, so nothing silently computes on the CPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libsbpmg.so"

SBP_OK = 0
SBP_ERR_ARGS = -1
SBP_ERR_CUDA = -2
SBP_ERR_NOMEM = -3
SBP_ERR_MAXITER = -4
SBP_ERR_BREAKDOWN = -5
SBP_ERR_UNSUPPORTED = -6
SBP_ERR_TIMEOUT = -7

SBP_SMOOTH_JACOBI = 0
SBP_SMOOTH_RICHARDSON = 1
SBP_RESTRICT_NORMAL = 0
SBP_RESTRICT_SBP = 1
SBP_RESTRICT_GALERKIN = 2
SBP_PREC_FP64 = 0
SBP_PREC_MIXED = 1


class sbp_options(C.Structure):
    _fields_ = [
        ("smoother", C.c_int),
        ("omega", C.c_double),
        ("nu_pre", C.c_int),
        ("nu_post", C.c_int),
        ("restriction", C.c_int),
        ("coarse_n", C.c_int),
        ("precision", C.c_int),
        ("reserved", C.c_int * 5),
    ]


class sbp_result(C.Structure):
    _fields_ = [
        ("iters", C.c_int),
        ("status", C.c_int),
        ("initial_norm", C.c_double),
        ("final_norm", C.c_double),
        ("threshold", C.c_double),
    ]


class sbp_kernel_time(C.Structure):
    _fields_ = [
        ("name", C.c_char * 160),
        ("launches", C.c_int),
        ("total_ms", C.c_double),
    ]


_vp = C.c_void_p
_i = C.c_int
_d = C.c_double
_dp = C.POINTER(C.c_double)

# name -> (restype, argtypes); every function of include/sbpmg.h
SIGNATURES = {
    "sbp_version": (_i, []),
    "sbp_status_string": (C.c_char_p, [_i]),
    "sbp_last_error": (C.c_char_p, []),
    "sbp_options_default": (None, [C.POINTER(sbp_options)]),
    "sbp_options_reference_two_level": (None, [C.POINTER(sbp_options), _i]),
    "sbp_apply_f64": (_i, [_vp, _vp, _i, _i, _vp]),
    "sbp_apply_f32": (_i, [_vp, _vp, _i, _i, _vp]),
    "sbp_apply_dot_f64": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "sbp_apply_dot_f64_noalloc": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "sbp_residual_norm_f64": (_i, [_vp, _vp, _i, _i, _dp, _vp]),
    "sbp_restrict_f64": (_i, [_vp, _vp, _i, _i, _vp]),
    "sbp_prolong_f64": (_i, [_vp, _vp, _i, _i, _vp]),
    "sbp_richardson_f64": (_i, [_vp, _vp, _vp, _i, _i, _d, _vp]),
    "sbp_jacobi_f64": (_i, [_vp, _vp, _vp, _i, _i, _d, _vp]),
    "sbp_rhs_f64": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _i, _d, _vp]),
    "sbp_rhs_adjoint_f64": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _i, _d, _vp]),
    "sbp_solver_create": (_i, [C.POINTER(_vp), _i, C.POINTER(sbp_options)]),
    "sbp_solver_destroy": (_i, [_vp]),
    "sbp_solver_levels": (_i, [_vp]),
    "sbp_solver_device_bytes": (C.c_longlong, [_vp]),
    "sbp_solver_last_launches": (C.c_longlong, [_vp]),
    "sbp_mgcg_solve": (_i, [_vp, _vp, _vp, _d, _d, _i, C.POINTER(sbp_result), _dp, _i, _vp]),
    "sbp_cg_solve": (_i, [_vp, _vp, _vp, _i, _d, _d, _i, C.POINTER(sbp_result), _dp, _i, _vp]),
    "sbp_vcycle_apply": (_i, [_vp, _vp, _vp, _vp]),
    "sbp_fp64_fma_rate": (_i, [_dp, _vp]),
    "sbp_test_drop_copy": (_i, [_i, C.c_uint]),
    "sbp_test_pair_to_f64": (_i, [_vp, _vp, _vp, C.c_longlong, _vp]),
    "sbp_solver_profile": (_i, [_vp, _i, _vp, _vp, _i, _d, _i, C.POINTER(sbp_result),
                                C.POINTER(sbp_kernel_time), _i, C.POINTER(_i), _vp]),
    "sbp_h_misfit_f64": (_i, [_vp, _vp, _vp, _i, _vp, _vp]),
    "sbp_mgcg_adjoint_f64": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _d, _i,
                                  C.POINTER(sbp_result), _vp]),
    "sbp_coarse_inverse_host": (_i, [_i, _dp, C.c_longlong]),
    "sbp_coarse_inverse_order_host": (_i, [_i, _i, _dp, C.c_longlong]),
    "sbp_apply_ho_f64": (_i, [_vp, _vp, _i, _i, _i, _vp]),
    "sbp_ho_solver_create": (_i, [C.POINTER(_vp), _i, _i, C.POINTER(sbp_options)]),
    "sbp_ho_solver_destroy": (_i, [_vp]),
    "sbp_ho_solver_levels": (_i, [_vp]),
    "sbp_ho_solver_device_bytes": (C.c_longlong, [_vp]),
    "sbp_ho_mgcg_solve": (_i, [_vp, _vp, _vp, _d, _d, _i, C.POINTER(sbp_result), _dp, _i, _vp]),
    "sbp_ho_cg_solve": (_i, [_vp, _vp, _vp, _i, _d, _d, _i, C.POINTER(sbp_result), _dp, _i,
                             _vp]),
    "sbp_ho_vcycle_apply": (_i, [_vp, _vp, _vp, _vp]),
    "sbp_apply_vc_f64": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "sbp_vc_solver_create": (_i, [C.POINTER(_vp), _i, _vp, C.POINTER(sbp_options)]),
    "sbp_vc_solver_destroy": (_i, [_vp]),
    "sbp_vc_solver_levels": (_i, [_vp]),
    "sbp_vc_solver_device_bytes": (C.c_longlong, [_vp]),
    "sbp_vc_mgcg_solve": (_i, [_vp, _vp, _vp, _d, _d, _i, C.POINTER(sbp_result), _dp, _i, _vp]),
    "sbp_vc_cg_solve": (_i, [_vp, _vp, _vp, _i, _d, _d, _i, C.POINTER(sbp_result), _dp, _i,
                             _vp]),
    "sbp_vc_vcycle_apply": (_i, [_vp, _vp, _vp, _vp]),
    "sbp_vc_coarsen_host": (_i, [_i, _dp, _dp]),
    "sbp_vc_galerkin_coarse_host": (_i, [_i, _dp, _dp, _dp, _dp, _dp, _dp]),
    "sbp_galerkin9_coarse_host": (_i, [_i] + [_dp] * 10),
    "sbp_vc_coarse_inverse_host": (_i, [_i, _dp, _dp, C.c_longlong]),
    "sbp_vc_assemble_host": (_i, [_i, _dp, C.POINTER(C.c_longlong), C.POINTER(_i), _dp,
                                  C.c_longlong, C.POINTER(C.c_longlong)]),
    "sbp_csr_assemble_host": (_i, [_i, C.POINTER(C.c_longlong), C.POINTER(_i), _dp,
                                   C.c_longlong, C.POINTER(C.c_longlong)]),
    "sbp_csr_spmv_f64": (_i, [C.c_longlong, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sbp_batch_create": (_i, [C.POINTER(_vp), C.POINTER(_i), _i, C.POINTER(sbp_options)]),
    "sbp_batch_destroy": (_i, [_vp]),
    "sbp_batch_size": (_i, [_vp]),
    "sbp_batch_device_bytes": (C.c_longlong, [_vp]),
    "sbp_batch_last_launches": (C.c_longlong, [_vp]),
    "sbp_batch_mgcg_solve": (_i, [_vp, C.POINTER(_vp), C.POINTER(_vp), _d, _d, _i,
                                  C.POINTER(sbp_result), _vp]),
    "sbp_batch_classes": (_i, [_vp, C.POINTER(_i), _i]),
    "sbp_batch_autotune": (_i, [_vp, C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_i), _vp]),
}

_lib = None


def load() -> C.CDLL:
    """Load libsbpmg.so (once) and attach the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python sc_2022_gb300/build.py`")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class SbpError(RuntimeError):
    """A libsbpmg call returned a negative status."""

    def __init__(self, status: int, where: str):
        lib = load()
        msg = lib.sbp_status_string(status).decode()
        if status in (SBP_ERR_CUDA, SBP_ERR_NOMEM, SBP_ERR_TIMEOUT):
            detail = lib.sbp_last_error().decode()
            if detail:
                msg = f"{msg} ({detail})"
        super().__init__(f"{where}: {msg} [status {status}]")
        self.status = status


def check(status: int, where: str) -> int:
    if status < 0:
        raise SbpError(status, where)
    return status
