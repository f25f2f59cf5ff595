"""ctypes binding of libdeo.so (the C ABI declared in include/deo.h).

This is the Python-side counterpart of the `ccall` stubs a Julia shim would
use.  The library is required: there is no CPU fallback, and importing this
module raises if libdeo.so has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "libdeo.so")

DEO_OK = 0
STATUS_NAMES = {0: "OK", 1: "BAD_SHAPE", 2: "BAD_ARG", 3: "UNSUPPORTED", 4: "CUDA", 5: "TIMEOUT", 6: "OOM",
                7: "NOT_READY", 8: "REJECTED"}
DEO_F64, DEO_F32 = 0, 1
DEO_BC_AFFINE, DEO_BC_PERIODIC = 0, 1
DEO_PATH_AUTO, DEO_PATH_PADDED, DEO_PATH_GENERIC = 0, 1, 2
DEO_OPT_FAST_PATH, DEO_OPT_TMA, DEO_OPT_EXACT_SUMS, DEO_OPT_LAUNCH_TIMING, DEO_OPT_CONCURRENT_SHELL = 1, 2, 3, 4, 5
DEO_OPT_FX_FP64_ROWS = 6
DEO_OPT_TEST_WITHHOLD = 7
DEO_OPT_F32_VECTOR = 8
DEO_OPT_SHELL_KERNEL = 9
DEO_OPT_F32_TILE = 10
DEO_PLAN_MERGE_TERMS = 1
DEO_PLAN_STAR = 2
DEO_PLAN_FACTOR_FIELD = 4
DEO_MAX_BC = 16

_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


class DeoError(RuntimeError):
    def __init__(self, status: int, msg: str):
        self.status = status
        super().__init__(f"deo {STATUS_NAMES.get(status, status)}: {msg}")


class DeoShapeError(DeoError, AssertionError):
    """Raised where the reference raises AssertionError / DimensionMismatch."""


class DeoArgError(DeoError, ValueError):
    """Raised where the reference raises ArgumentError / AssertionError on arguments."""


class OperatorDesc(C.Structure):
    _fields_ = [("derivative_order", C.c_int), ("approximation_order", C.c_int), ("len", C.c_int),
                ("stencil_length", C.c_int), ("boundary_stencil_length", C.c_int),
                ("boundary_point_count", C.c_int), ("offside", C.c_int), ("winding", C.c_int),
                ("uniform", C.c_int), ("coeff_func_sign", C.c_int), ("n_stencil_rows", C.c_int),
                ("n_low_rows", C.c_int), ("n_high_rows", C.c_int),
                ("stencil_coefs", _dp), ("low_boundary_coefs", _dp), ("high_boundary_coefs", _dp),
                ("coefficients", _dp)]


class BCStruct(C.Structure):
    _fields_ = [("kind", C.c_int), ("m_l", C.c_int), ("m_r", C.c_int),
                ("a_l", C.c_double * DEO_MAX_BC), ("a_r", C.c_double * DEO_MAX_BC),
                ("b_l", C.c_double), ("b_r", C.c_double)]


class Term(C.Structure):
    _fields_ = [("op", _vp), ("axis", C.c_int), ("bc", C.POINTER(BCStruct)), ("coeff_field", _vp),
                ("path", C.c_int), ("line_bcs", C.POINTER(BCStruct))]


class Request(C.Structure):
    _fields_ = [("plan", _vp), ("u0", _vp), ("nsteps", C.c_int), ("dt", C.c_double), ("want_grad", C.c_int)]


class ServeStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "admitted", "completed", "rejected", "failed", "cancelled",
                                          "rounds", "steps", "launches", "rebuilds", "in_use_bytes", "active",
                                          "pending", "device_us")]


class Instance(C.Structure):
    _fields_ = [("plan", _vp), ("u", _vp), ("du", _vp)]


class Stage(C.Structure):
    _fields_ = [("plan", _vp), ("a", _vp), ("b", _vp), ("c", _vp), ("out", _vp),
                ("alpha", C.c_double), ("beta", C.c_double), ("gamma", C.c_double), ("dt", C.c_double),
                ("adjoint", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libdeo.so not found at {LIB_PATH}; build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(LIB_PATH)
    st = C.c_int

    def proto(name, res, *args):
        f = getattr(L, name)
        f.restype = res
        f.argtypes = list(args)

    proto("deo_last_error", C.c_char_p)
    proto("deo_abi_version", C.c_int)
    proto("deo_calculate_weights", st, C.c_int, C.c_double, _dp, C.c_int, _dp)
    proto("deo_centered_difference", st, C.c_int, C.c_int, _dp, C.c_int, C.c_int, C.POINTER(_vp))
    proto("deo_upwind_difference", st, C.c_int, C.c_int, _dp, C.c_int, C.c_int, C.c_int, C.POINTER(_vp))
    proto("deo_operator_from_tables", st, C.POINTER(OperatorDesc), C.POINTER(_vp))
    proto("deo_operator_describe", st, _vp, C.POINTER(OperatorDesc))
    proto("deo_operator_set_coefficients", st, _vp, _dp, C.c_int, C.c_int)
    proto("deo_operator_scale_coefficients", st, _vp, _dp, C.c_int)
    proto("deo_operator_clone", st, _vp, C.POINTER(_vp))
    proto("deo_operator_destroy", None, _vp)
    proto("deo_operator_array", st, _vp, _dp)
    proto("deo_operator_banded", st, _vp, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp)
    proto("deo_robin_bc", st, _dp, _dp, _dp, C.c_int, C.c_int, C.POINTER(BCStruct))
    proto("deo_general_bc", st, _dp, C.c_int, _dp, C.c_int, _dp, C.c_int, C.c_int, C.POINTER(BCStruct))
    proto("deo_dirichlet_bc", st, C.c_double, C.c_double, C.POINTER(BCStruct))
    proto("deo_neumann_bc", st, C.c_double, C.c_double, _dp, C.c_int, C.c_int, C.POINTER(BCStruct))
    proto("deo_periodic_bc", st, C.POINTER(BCStruct))
    proto("deo_bc_array", st, C.POINTER(BCStruct), C.c_int, _dp, _dp)
    proto("deo_plan_create", st, C.c_int, C.POINTER(C.c_int64), C.c_int, C.c_int, C.POINTER(Term), C.POINTER(_vp))
    proto("deo_plan_terms", C.c_int, _vp)
    proto("deo_plan_star_taps", C.c_int, _vp)
    proto("deo_plan_create_opts", st, C.c_int, C.POINTER(C.c_int64), C.c_int, C.c_int, C.POINTER(Term), C.c_int,
          C.POINTER(_vp))
    proto("deo_plan_destroy", None, _vp)
    proto("deo_plan_table_bytes", C.c_size_t, _vp)
    proto("deo_plan_set_option", st, _vp, C.c_int, C.c_int)
    proto("deo_plan_get_option", C.c_int, _vp, C.c_int)
    proto("deo_plan_kernels", C.c_char_p, _vp, C.c_int)
    proto("deo_plan_launch_times", C.c_int, _vp, C.POINTER(C.c_float), C.POINTER(C.c_int))
    proto("deo_device_status", st, C.POINTER(C.c_uint))
    proto("deo_apply", st, _vp, _vp, _vp, C.c_int, _vp)
    proto("deo_apply_host", st, _vp, _vp, _vp, _vp)
    proto("deo_nonlinear_diffusion_plan", st, C.c_int, C.c_int, C.c_int, _dp, C.c_int, C.c_int, C.c_int,
          C.POINTER(_vp))
    proto("deo_nonlinear_diffusion", st, _vp, _vp, _vp, _vp, _vp)
    proto("deo_nonlinear_diffusion_destroy", None, _vp)
    proto("deo_padded_plan", st, _vp, C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int,
          C.POINTER(_vp))
    proto("deo_padded_plan_view", st, _vp, C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
          C.POINTER(C.c_int64), C.c_int, C.POINTER(_vp))
    proto("deo_padded_apply", st, _vp, _vp, _vp, C.c_int, _vp)
    proto("deo_padded_destroy", None, _vp)
    proto("deo_solve_plan", st, _vp, _vp, C.c_int, C.POINTER(C.c_int64), C.c_int, C.c_int, C.POINTER(_vp))
    proto("deo_solve_bands", st, _vp, C.POINTER(C.c_int), C.POINTER(C.c_int))
    proto("deo_solve_apply", st, _vp, _vp, _vp, _vp)
    proto("deo_solve_destroy", None, _vp)
    proto("deo_vector_calculus_plan", st, C.c_int, C.c_int, C.POINTER(_vp), C.c_int, C.POINTER(_vp))
    proto("deo_vector_calculus_sizes", st, _vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64))
    proto("deo_vector_calculus_apply", st, _vp, _vp, _vp, C.c_int, _vp)
    proto("deo_vector_calculus_info", st, _vp, C.POINTER(C.c_int))
    proto("deo_vector_calculus_destroy", None, _vp)
    proto("deo_dot_product", st, C.c_int, C.c_int64, C.c_int, _vp, _vp, _vp, _vp)
    proto("deo_cross_product", st, C.c_int, C.c_int64, _vp, _vp, _vp, _vp)
    proto("deo_square_norm", st, C.c_int, C.c_int64, C.c_int, _vp, _vp, _vp)
    proto("deo_apply_host_async", st, _vp, _vp, _vp, _vp)
    proto("deo_plan_host_sync", st, _vp)
    proto("deo_apply_adjoint", st, _vp, _vp, _vp, C.c_int, _vp)
    proto("deo_plan_concretize", st, _vp, _dp, _dp)
    proto("deo_plan_concretize_device", st, _vp, _vp, _vp, _vp)
    proto("deo_plan_bandwidths", st, _vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _vp)
    proto("deo_plan_concretize_banded", st, _vp, C.c_int64, C.c_int64, _vp, _vp, _vp)
    proto("deo_batch_create", st, C.c_int, C.POINTER(Instance), C.c_int, C.c_int, C.c_int, C.POINTER(_vp))
    proto("deo_stage_batch_create", st, C.c_int, C.POINTER(Stage), C.c_int, C.c_int, C.POINTER(_vp))
    proto("deo_batch_run", st, _vp, C.c_int, _vp)
    proto("deo_apply_each", st, C.c_int, C.POINTER(Instance), C.c_int, _vp)
    proto("deo_batch_apply_noalloc", st, C.c_int, C.POINTER(Instance), C.c_int, C.c_int, _vp)
    proto("deo_batch_set_buffers", st, _vp, C.c_int, _vp, _vp)
    proto("deo_batch_config", st, _vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64))
    proto("deo_batch_destroy", None, _vp)
    proto("deo_batch_autotune", st, _vp, C.c_char_p, _vp)
    proto("deo_plan_autotune", st, _vp, _vp, _vp, C.c_char_p, _vp)
    proto("deo_plan_autotune_times", st, _vp, C.POINTER(C.c_int), C.POINTER(C.c_float), C.c_int,
          C.POINTER(C.c_int))
    proto("deo_serve_create", st, C.c_size_t, C.c_int, C.c_int, C.POINTER(_vp))
    proto("deo_serve_submit", st, _vp, C.POINTER(Request), C.POINTER(C.c_int64))
    proto("deo_serve_pump", st, _vp)
    proto("deo_serve_poll", st, _vp, C.c_int64, _vp, _vp, C.POINTER(C.c_double))
    proto("deo_serve_cancel", st, _vp, C.c_int64)
    proto("deo_serve_stats_get", st, _vp, C.POINTER(ServeStats))
    proto("deo_serve_inject_alloc_failures", st, _vp, C.c_int)
    proto("deo_serve_destroy", None, _vp)
    _lib = L
    return L


def check(status: int) -> None:
    if status == DEO_OK:
        return
    msg = lib().deo_last_error().decode(errors="replace")
    if status == 1:
        raise DeoShapeError(status, msg)
    if status == 2:
        raise DeoArgError(status, msg)
    raise DeoError(status, msg)


# Every symbol include/deo.h declares (checked by the CPU test-suite).
EXPORTED = [
    "deo_last_error", "deo_abi_version", "deo_calculate_weights", "deo_centered_difference",
    "deo_upwind_difference", "deo_operator_from_tables", "deo_operator_describe",
    "deo_operator_set_coefficients", "deo_operator_scale_coefficients", "deo_operator_clone",
    "deo_operator_destroy", "deo_operator_array", "deo_operator_banded", "deo_robin_bc", "deo_general_bc", "deo_dirichlet_bc",
    "deo_neumann_bc", "deo_periodic_bc", "deo_bc_array", "deo_plan_create", "deo_plan_create_opts", "deo_plan_terms", "deo_plan_star_taps", "deo_plan_destroy",
    "deo_plan_table_bytes", "deo_plan_set_option", "deo_plan_get_option", "deo_plan_kernels", "deo_plan_launch_times", "deo_device_status", "deo_apply", "deo_apply_host", "deo_nonlinear_diffusion_plan", "deo_nonlinear_diffusion",
    "deo_nonlinear_diffusion_destroy", "deo_apply_host_async", "deo_plan_host_sync", "deo_apply_adjoint", "deo_plan_concretize", "deo_plan_concretize_device", "deo_plan_bandwidths",
    "deo_plan_concretize_banded",
    "deo_batch_create", "deo_stage_batch_create", "deo_batch_run", "deo_apply_each", "deo_batch_apply_noalloc", "deo_batch_set_buffers", "deo_batch_config", "deo_batch_destroy",
    "deo_serve_create", "deo_serve_submit", "deo_serve_pump", "deo_serve_poll", "deo_serve_cancel", "deo_serve_stats_get",
    "deo_serve_inject_alloc_failures", "deo_serve_destroy",
    "deo_batch_autotune", "deo_plan_autotune", "deo_plan_autotune_times", "deo_vector_calculus_plan", "deo_vector_calculus_sizes", "deo_vector_calculus_apply", "deo_vector_calculus_info",
    "deo_vector_calculus_destroy", "deo_dot_product", "deo_cross_product", "deo_square_norm",
    "deo_solve_plan", "deo_solve_bands", "deo_solve_apply", "deo_solve_destroy",
    "deo_padded_plan", "deo_padded_plan_view", "deo_padded_apply", "deo_padded_destroy",
]
