"""ctypes binding of include/mpart_gb300.h.  Loads the in-tree
libmpart_gb300.so and fails loudly when it is missing: there is no CPU
fallback for the product path."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmpart_gb300.so")

MPGB_OK = 0
MPGB_ERR_INVALID_ARGUMENT = -1
MPGB_ERR_RUNTIME = -2
MPGB_ERR_CUDA = -3
MPGB_ERR_INTEGRAND = -4


class mpgb_map_options(C.Structure):
    _fields_ = [
        ("basis_type", C.c_int),
        ("pos_func_type", C.c_int),
        ("quad_type", C.c_int),
        ("quad_abs_tol", C.c_double),
        ("quad_rel_tol", C.c_double),
        ("quad_max_sub", C.c_uint),
        ("quad_min_sub", C.c_uint),
        ("quad_pts", C.c_uint),
        ("cont_deriv", C.c_int),
        ("basis_norm", C.c_int),
        ("nugget", C.c_double),
        ("sigmoid_type", C.c_int),
        ("edge_type", C.c_int),
        ("edge_shape", C.c_double),
        ("sigmoid_sum_type", C.c_int),
    ]


class mpgb_matrix(C.Structure):
    _fields_ = [
        ("data", C.c_void_p),
        ("rows", C.c_int64),
        ("cols", C.c_int64),
        ("row_stride", C.c_int64),
        ("col_stride", C.c_int64),
    ]


class mpgb_train_options(C.Structure):
    _fields_ = [("max_iters", C.c_int), ("max_evals", C.c_int), ("ftol_rel", C.c_double), ("ftol_abs", C.c_double),
                ("xtol_rel", C.c_double), ("xtol_abs", C.c_double), ("gtol", C.c_double), ("memory", C.c_int),
                ("mode", C.c_int), ("algorithm", C.c_int), ("precondition", C.c_int)]


class mpgb_train_result(C.Structure):
    _fields_ = [("total_loss", C.c_double), ("iterations", C.c_int), ("evaluations", C.c_int), ("steps", C.c_int),
                ("ms_per_step", C.c_double), ("total_ms", C.c_double), ("grad_norm", C.c_double)]


class mpgb_atm_options(C.Structure):
    _fields_ = [("map", mpgb_map_options), ("train", mpgb_train_options), ("max_patience", C.c_uint),
                ("max_size", C.c_uint), ("max_degrees", C.POINTER(C.c_uint)), ("verbose", C.c_int)]


class mpgb_atm_result(C.Structure):
    _fields_ = [("size", C.c_uint), ("iterations", C.c_uint), ("best_test_error", C.c_double),
                ("final_train_error", C.c_double), ("final_test_error", C.c_double), ("total_ms", C.c_double)]


# Every symbol the header declares, with its signature.
_MAP = C.c_void_p
_MAPP = C.POINTER(C.c_void_p)
_UP = C.POINTER(C.c_uint)
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    "mpgb_version": (C.c_char_p, []),
    "mpgb_last_error": (C.c_char_p, []),
    "mpgb_map_options_default": (C.c_int, [C.POINTER(mpgb_map_options)]),
    "mpgb_create_component": (C.c_int, [C.c_uint, C.c_uint, _UP, _UP, _UP, C.POINTER(mpgb_map_options), _MAPP]),
    "mpgb_create_component_total_order": (C.c_int, [C.c_uint, C.c_uint, C.POINTER(mpgb_map_options), _MAPP]),
    "mpgb_create_triangular": (C.c_int, [C.c_uint, C.c_uint, C.c_uint, C.POINTER(mpgb_map_options), _MAPP]),
    "mpgb_create_triangular_from_components": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint, C.c_int, _MAPP]),
    "mpgb_create_sigmoid_component": (C.c_int, [C.c_uint, C.c_uint, C.c_uint, _DP, C.c_uint,
                                                C.POINTER(mpgb_map_options), _MAPP]),
    "mpgb_create_sigmoid_component_mset": (C.c_int, [C.c_uint, C.c_uint, _UP, _UP, _UP, _DP, C.c_uint,
                                                     C.POINTER(mpgb_map_options), _MAPP]),
    "mpgb_create_sigmoid_triangular": (C.c_int, [C.c_uint, C.c_uint, C.c_uint, _DP, C.c_uint, C.c_int64,
                                                 C.c_int64, C.POINTER(mpgb_map_options), _MAPP]),
    "mpgb_map_coeff_bounds": (C.c_int, [_MAP, _DP, _DP]),
    "mpgb_map_kind": (C.c_int, [_MAP, C.POINTER(C.c_int)]),
    "mpgb_component_sigmoid": (C.c_int, [_MAP, _DP, _DP, _DP, _UP, _UP, _UP]),
    "mpgb_sigmoid_params": (C.c_int, [_DP, C.c_uint, C.c_double, C.c_int, _DP, _DP, _DP, _UP, _UP]),
    "mpgb_sigmoid1d_evaluate": (C.c_int, [_DP, _DP, _DP, C.c_uint, _UP, C.c_uint, C.c_int, C.c_uint, C.c_void_p,
                                          C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mpgb_map_destroy": (C.c_int, [_MAP]),
    "mpgb_map_dims": (C.c_int, [_MAP, _UP, _UP, _UP]),
    "mpgb_map_num_components": (C.c_int, [_MAP, _UP]),
    "mpgb_map_get_component": (C.c_int, [_MAP, C.c_uint, _MAPP]),
    "mpgb_set_coeffs": (C.c_int, [_MAP, C.c_void_p, C.c_uint, C.c_int, C.c_void_p]),
    "mpgb_wrap_coeffs": (C.c_int, [_MAP, C.c_void_p, C.c_uint]),
    "mpgb_get_coeffs": (C.c_int, [_MAP, C.c_void_p, C.c_uint]),
    "mpgb_coeffs_device_ptr": (C.c_int, [_MAP, C.POINTER(C.c_void_p)]),
    "mpgb_set_async": (C.c_int, [_MAP, C.c_int]),
    "mpgb_set_point_ordering": (C.c_int, [_MAP, C.c_int]),
    "mpgb_check_status": (C.c_int, [_MAP, C.c_void_p, C.POINTER(C.c_int)]),
    "mpgb_evaluate": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, C.c_void_p]),
    "mpgb_log_determinant": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, C.c_void_p]),
    "mpgb_inverse": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, mpgb_matrix, C.c_double, C.c_double, C.c_void_p,
                               C.c_void_p]),
    "mpgb_inverse_method": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, mpgb_matrix, C.c_double, C.c_double, C.c_int,
                                      C.c_void_p, C.c_void_p]),
    "mpgb_coeff_grad": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, mpgb_matrix, C.c_void_p]),
    "mpgb_gradient": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, mpgb_matrix, C.c_void_p]),
    "mpgb_log_determinant_coeff_grad": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, C.c_void_p]),
    "mpgb_log_determinant_input_grad": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, C.c_void_p]),
    "mpgb_fused_fwd_adj": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, mpgb_matrix, C.c_double, mpgb_matrix,
                                     mpgb_matrix, C.c_void_p, mpgb_matrix, C.c_void_p]),
    "mpgb_fused_fwd_adj_noalloc": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, mpgb_matrix, C.c_double, mpgb_matrix,
                                             mpgb_matrix, C.c_void_p, C.c_void_p]),
    "mpgb_kl_objective": (C.c_int, [_MAP, mpgb_matrix, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mpgb_inverse_coeff_grad": (C.c_int, [_MAP, mpgb_matrix, mpgb_matrix, C.c_void_p, mpgb_matrix, C.c_void_p]),
    "mpgb_fp64_probe": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_float)]),
    "mpgb_launch_count": (C.c_longlong, []),
    "mpgb_atm_options_default": (C.c_int, [C.POINTER(mpgb_atm_options)]),
    "mpgb_train_map_adaptive": (C.c_int, [C.c_uint, _UP, _UP, mpgb_matrix, mpgb_matrix, C.POINTER(mpgb_atm_options),
                                          _MAPP, C.POINTER(mpgb_atm_result), _UP, C.c_void_p]),
    "mpgb_reduced_margin": (C.c_int, [C.c_uint, C.c_uint, _UP, _UP, _UP, C.c_uint]),
    "mpgb_multi_index_expand": (C.c_int, [C.c_uint, C.c_uint, _UP, _UP, _UP, _UP, _UP, C.c_uint]),
    "mpgb_optimizer_self_test": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _DP, _DP, _DP, C.POINTER(C.c_int),
                                           C.POINTER(C.c_int)]),
    "mpgb_component_multi_index": (C.c_int, [_MAP, _UP, _UP, _UP, _UP, _UP, _UP]),
    "mpgb_map_is_triangular": (C.c_int, [_MAP, C.POINTER(C.c_int)]),
    "mpgb_map_to_bytes": (C.c_int, [_MAP, C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "mpgb_map_from_bytes": (C.c_int, [C.c_void_p, C.c_size_t, _MAPP]),
    "mpgb_map_archive_rewrite": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "mpgb_coeff_archive_read": (C.c_int, [C.c_void_p, C.c_size_t, _UP, _UP, _UP, C.c_void_p]),
    "mpgb_options_to_bytes": (C.c_int, [C.POINTER(mpgb_map_options), C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "mpgb_options_from_bytes": (C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(mpgb_map_options)]),
    "mpgb_mset_to_bytes": (C.c_int, [C.c_uint, C.c_uint, _UP, _UP, _UP, C.c_void_p, C.c_size_t,
                                     C.POINTER(C.c_size_t)]),
    "mpgb_mset_from_bytes": (C.c_int, [C.c_void_p, C.c_size_t, _UP, _UP, _UP, _UP, _UP, _UP]),
    "mpgb_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "mpgb_batch_destroy": (C.c_int, [C.c_void_p]),
    "mpgb_batch_fwd_adj": (C.c_int, [C.c_void_p, C.POINTER(mpgb_matrix), C.POINTER(mpgb_matrix), C.c_double,
                                     C.POINTER(mpgb_matrix), C.POINTER(mpgb_matrix), C.POINTER(C.c_void_p),
                                     C.c_void_p]),
    "mpgb_batch_autotune": (C.c_int, [C.c_void_p, C.POINTER(mpgb_matrix), C.POINTER(mpgb_matrix), C.c_double, C.c_int,
                                      C.POINTER(C.c_double), C.c_void_p]),
    "mpgb_batch_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mpgb_batch_set_tuning": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int)]),
    "mpgb_train_options_default": (C.c_int, [C.POINTER(mpgb_train_options)]),
    "mpgb_train_map": (C.c_int, [_MAP, mpgb_matrix, C.POINTER(mpgb_train_options), C.c_void_p,
                                 C.POINTER(mpgb_train_result), C.c_void_p]),
    "mpgb_kl_step_time": (C.c_int, [_MAP, mpgb_matrix, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_void_p,
                                    C.c_void_p, C.c_void_p]),
    "mpgb_plain_create": (C.c_int, [C.c_uint, C.c_uint, C.POINTER(mpgb_map_options), _MAPP]),
    "mpgb_plain_destroy": (C.c_int, [_MAP]),
    "mpgb_plain_num_terms": (C.c_int, [_MAP, _UP]),
    "mpgb_plain_fwd_adj": (C.c_int, [_MAP, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p]),
}

_lib = None


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"libmpart_gb300.so not found at {LIB_PATH}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class MpgbError(RuntimeError):
    pass


class IntegrandError(MpgbError):
    pass


def check(rc: int):
    if rc == MPGB_OK:
        return
    msg = load().mpgb_last_error().decode(errors="replace")
    if rc == MPGB_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    if rc == MPGB_ERR_INTEGRAND:
        raise IntegrandError(msg)
    raise MpgbError(msg)
