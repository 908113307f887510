"""ctypes binding of libtk_heff.so (declarations in include/tk_heff.h).

The library is loaded from this package directory only; if it is missing the
import fails loudly (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libtk_heff.so"

TK_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "SECTOR_MISMATCH", 3: "OOM", 4: "CUDA", 5: "TIMEOUT",
                6: "CANCELLED", 7: "UNSUPPORTED"}
PREC_FP64, PREC_BF16X3 = 0, 1
SCHED_GROUPED, SCHED_PER_BLOCK, SCHED_STACKED = 0, 1, 2
HOST_IO_STAGED, HOST_IO_DIRECT, HOST_IO_DIRECT_OUT, HOST_IO_AUTO = 0, 1, 2, 3


class TkError(RuntimeError):
    """Failure reported by the C ABI (status code + tk_last_error message)."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class tk_qindex(C.Structure):
    _fields_ = [("n_sectors", C.c_int32), ("charges", C.POINTER(C.c_int32)), ("dims", C.POINTER(C.c_int64))]


class tk_bst(C.Structure):
    _fields_ = [("qn_kind", C.c_int32), ("rank", C.c_int32), ("legs", C.POINTER(tk_qindex)),
                ("leg_dirs", C.POINTER(C.c_int8)), ("flux", C.POINTER(C.c_int32)), ("n_blocks", C.c_int64),
                ("keys", C.POINTER(C.c_uint64)), ("block_offsets", C.POINTER(C.c_int64)),
                ("data", C.POINTER(C.c_double))]


class tk_env(C.Structure):
    _fields_ = [("bra", tk_qindex), ("mpo", tk_qindex), ("ket", tk_qindex), ("data", C.POINTER(C.c_double))]


class tk_lanczos_cfg(C.Structure):
    _fields_ = [("krylov_dim", C.c_int32), ("max_restarts", C.c_int32), ("tol", C.c_double),
                ("refine", C.c_int32)]


class tk_davidson_cfg(C.Structure):
    _fields_ = [("max_subspace", C.c_int32), ("max_iter", C.c_int32), ("tol", C.c_double),
                ("diagonal", C.c_void_p), ("inner", C.c_int32)]


class tk_expm_cfg(C.Structure):
    _fields_ = [("krylov_dim", C.c_int32), ("tol", C.c_double)]


class tk_expm_result(C.Structure):
    _fields_ = [("krylov_used", C.c_int32), ("matvec_count", C.c_int32), ("input_norm", C.c_double)]


class tk_eigen_result(C.Structure):
    _fields_ = [("eigenvalue", C.c_double), ("residual_norm", C.c_double), ("converged", C.c_int32),
                ("matvec_count", C.c_int32), ("fp64_matvec_count", C.c_int32), ("restarts", C.c_int32)]


class tk_mat(C.Structure):
    _fields_ = [("data", C.c_void_p), ("rows", C.c_int64), ("cols", C.c_int64), ("row_stride", C.c_int64),
                ("col_stride", C.c_int64), ("is_conjugated", C.c_int32)]


class tk_cmat(C.Structure):
    _fields_ = [("re", C.c_void_p), ("im", C.c_void_p), ("rows", C.c_int64), ("cols", C.c_int64),
                ("row_stride", C.c_int64), ("col_stride", C.c_int64), ("is_conjugated", C.c_int32)]


class tk_mat_mut(C.Structure):
    _fields_ = [("data", C.c_void_p), ("rows", C.c_int64), ("cols", C.c_int64), ("row_stride", C.c_int64),
                ("col_stride", C.c_int64)]


class tk_tc_options(C.Structure):
    _fields_ = [("tall_max_mtiles", C.c_int32), ("fuse_max_ntiles", C.c_int32), ("combine_warps", C.c_int32),
                ("stage1_persistent", C.c_int32), ("stage1_narrow", C.c_int32)]


class tk_autotune_result(C.Structure):
    _fields_ = [("chosen", tk_tc_options), ("chosen_ms", C.c_float), ("from_cache", C.c_int32),
                ("n_candidates", C.c_int32), ("candidates", tk_tc_options * 8), ("candidate_ms", C.c_float * 8)]


class tk_bst_out(C.Structure):
    _fields_ = [("qn_kind", C.c_int32), ("rank", C.c_int32), ("legs", tk_qindex * 2), ("leg_dirs", C.c_int8 * 2),
                ("flux", C.c_int32 * 2), ("n_blocks", C.c_int64), ("keys", C.POINTER(C.c_uint64)),
                ("block_offsets", C.POINTER(C.c_int64)), ("data", C.POINTER(C.c_double)), ("total", C.c_int64),
                ("owned_charges", C.POINTER(C.c_int32)), ("owned_dims", C.POINTER(C.c_int64))]


# (name, restype, argtypes) of every entry point declared in include/tk_heff.h
SIGNATURES = [
    ("tk_version", C.c_int32, []),
    ("tk_last_error", C.c_char_p, []),
    ("tk_ctx_create", C.c_int32, [C.c_int32, C.POINTER(C.c_void_p)]),
    ("tk_ctx_destroy", None, [C.c_void_p]),
    ("tk_heff2_plan_create", C.c_int32, [C.c_void_p, C.POINTER(tk_env), C.POINTER(tk_env), C.POINTER(tk_bst),
                                         C.POINTER(tk_bst), C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_void_p)]),
    ("tk_heff2_plan_destroy", None, [C.c_void_p]),
    ("tk_heff2_plan_footprint", C.c_int32, [C.POINTER(tk_env), C.POINTER(tk_env), C.POINTER(tk_bst),
                                            C.POINTER(tk_bst), C.POINTER(C.c_int32), C.c_int32,
                                            C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("tk_debug_fail_host_alloc", None, [C.c_int32]),
    ("tk_debug_fail_device_alloc", None, [C.c_int32]),
    ("tk_heff2_set_cancel_flag", C.c_int32, [C.c_void_p, C.c_void_p]),
    ("tk_heff2_set_tc_options", C.c_int32, [C.c_void_p, C.POINTER(tk_tc_options)]),
    ("tk_heff2_get_tc_options", C.c_int32, [C.c_void_p, C.POINTER(tk_tc_options)]),
    ("tk_heff2_autotune", C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(tk_autotune_result)]),
    ("tk_heff2_inject_error_word", C.c_int32, [C.c_void_p, C.c_int32]),
    ("tk_heff2_dims", C.c_int32, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("tk_heff2_blocks", C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_int64)]),
    ("tk_heff2_cost", C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("tk_heff2_launches", C.c_int32, [C.c_void_p, C.POINTER(C.c_int32)]),
    ("tk_heff2_set_host_io", C.c_int32, [C.c_void_p, C.c_int32]),
    ("tk_heff2_set_precision", C.c_int32, [C.c_void_p, C.c_int32]),
    ("tk_heff2_set_schedule", C.c_int32, [C.c_void_p, C.c_int32]),
    ("tk_heff2_set_psi_pieces", C.c_int32, [C.c_void_p, C.c_int32]),
    ("tk_heff2_get_schedule", C.c_int32, [C.c_void_p, C.POINTER(C.c_int32)]),
    ("tk_heff2_profile", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                     C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("tk_heff2_apply", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_heff2_apply_host", C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("tk_heff2_apply_host_flat", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_heff2_dense_to_flat", C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("tk_heff2_flat_to_dense", C.c_int32, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("tk_lanczos_lowest", C.c_int32, [C.c_void_p, C.POINTER(tk_lanczos_cfg), C.c_void_p, C.c_void_p,
                                      C.POINTER(tk_eigen_result), C.c_void_p]),
    ("tk_davidson_lowest", C.c_int32, [C.c_void_p, C.POINTER(tk_davidson_cfg), C.c_void_p, C.c_void_p,
                                       C.POINTER(tk_eigen_result), C.c_void_p]),
    ("tk_expm_krylov", C.c_int32, [C.c_void_p, C.POINTER(tk_expm_cfg), C.c_double, C.c_double, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(tk_expm_result), C.c_void_p]),
    ("tk_gemm_f64", C.c_int32, [C.c_void_p, C.c_double, C.POINTER(tk_mat), C.POINTER(tk_mat), C.c_double,
                                C.POINTER(tk_mat_mut), C.c_void_p]),
    ("tk_gemm_f64_noalloc", C.c_int32, [C.c_void_p, C.c_double, C.POINTER(tk_mat), C.POINTER(tk_mat), C.c_double,
                                        C.POINTER(tk_mat_mut), C.c_void_p]),
    ("tk_block_gemm_f64", C.c_int32, [C.c_void_p, C.POINTER(tk_bst), C.POINTER(tk_bst), C.POINTER(tk_bst_out)]),
    ("tk_bst_free", None, [C.POINTER(tk_bst_out)]),
    ("tk_block_gemm_f64_dev", C.c_int32, [C.c_void_p, C.POINTER(tk_bst), C.POINTER(tk_bst), C.POINTER(tk_bst_out),
                                          C.c_void_p, C.c_void_p]),
    ("tk_contract_pairwise_f64", C.c_int32, [C.c_void_p, C.POINTER(tk_bst), C.POINTER(C.c_int32), C.c_int32,
                                             C.POINTER(tk_bst), C.POINTER(C.c_int32), C.c_int32,
                                             C.POINTER(tk_bst_out)]),
    ("tk_spmv_f64", C.c_int32, [C.c_void_p, C.POINTER(tk_bst), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("tk_heff2_plan_create_dev_complex", C.c_int32, [C.c_void_p, C.POINTER(tk_env), C.c_void_p, C.POINTER(tk_env),
                                                     C.c_void_p, C.POINTER(tk_bst), C.POINTER(tk_bst),
                                                     C.POINTER(C.c_int32), C.POINTER(C.c_void_p)]),
    ("tk_heff2_apply_complex", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_env_grow_left_complex", C.c_int32, [C.c_void_p, C.POINTER(tk_env), C.c_void_p, C.POINTER(tk_bst),
                                             C.c_void_p, C.POINTER(tk_bst), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_env_grow_right_complex", C.c_int32, [C.c_void_p, C.POINTER(tk_env), C.c_void_p, C.POINTER(tk_bst),
                                              C.c_void_p, C.POINTER(tk_bst), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_heff2_two_site_product_complex", C.c_int32, [C.c_void_p, C.POINTER(tk_bst), C.c_void_p, C.POINTER(tk_bst),
                                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_svd_truncated_f64", C.c_int32, [C.c_void_p, C.POINTER(tk_mat), C.c_int64, C.c_double, C.c_void_p,
                                         C.POINTER(C.c_double), C.c_void_p, C.POINTER(C.c_int64),
                                         C.POINTER(C.c_double), C.c_void_p]),
    ("tk_eigh_lowest_f64", C.c_int32, [C.c_void_p, C.POINTER(tk_mat), C.c_int64, C.POINTER(C.c_double), C.c_void_p,
                                       C.c_void_p]),
    ("tk_eigh_batched_f64", C.c_int32, [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_qr_f64", C.c_int32, [C.c_void_p, C.POINTER(tk_mat), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_svd_truncated_c64", C.c_int32, [C.c_void_p, C.POINTER(tk_cmat), C.c_int64, C.c_double, C.c_void_p,
                                         C.c_void_p, C.POINTER(C.c_double), C.c_void_p, C.c_void_p,
                                         C.POINTER(C.c_int64), C.POINTER(C.c_double), C.c_void_p]),
    ("tk_eigh_lowest_c64", C.c_int32, [C.c_void_p, C.POINTER(tk_cmat), C.c_int64, C.POINTER(C.c_double),
                                       C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_qr_c64", C.c_int32, [C.c_void_p, C.POINTER(tk_cmat), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p]),
    ("tk_check_split_conversions", C.c_int32, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_uint64)]),
    ("tk_env_layout", C.c_int32, [C.c_int32, C.POINTER(tk_qindex), C.POINTER(tk_qindex), C.POINTER(tk_qindex),
                                  C.POINTER(C.c_int64), C.POINTER(C.c_uint64), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int64)]),
    ("tk_heff2_plan_create_dev", C.c_int32, [C.c_void_p, C.POINTER(tk_env), C.POINTER(tk_env), C.POINTER(tk_bst),
                                             C.POINTER(tk_bst), C.POINTER(C.c_int32), C.c_int32,
                                             C.POINTER(C.c_void_p)]),
    ("tk_env_grow_left", C.c_int32, [C.c_void_p, C.POINTER(tk_env), C.POINTER(tk_bst), C.POINTER(tk_bst),
                                     C.c_void_p, C.c_void_p]),
    ("tk_env_grow_right", C.c_int32, [C.c_void_p, C.POINTER(tk_env), C.POINTER(tk_bst), C.POINTER(tk_bst),
                                      C.c_void_p, C.c_void_p]),
    ("tk_heff2_two_site_product", C.c_int32, [C.c_void_p, C.POINTER(tk_bst), C.POINTER(tk_bst), C.c_void_p,
                                              C.c_void_p]),
    ("tk_split_plan_create", C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(tk_qindex), C.c_int64,
                                         C.POINTER(C.c_uint64), C.POINTER(C.c_int64), C.POINTER(C.c_void_p)]),
    ("tk_split_plan_destroy", None, [C.c_void_p]),
    ("tk_split_charges", C.c_int32, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                     C.POINTER(C.c_int64)]),
    ("tk_split_gather", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("tk_split_set_kept", C.c_int32, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("tk_split_layout", C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_uint64), C.POINTER(C.c_int64)]),
    ("tk_split_factors", C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
]

_lib = None


def load() -> C.CDLL:
    """Loads libtk_heff.so and binds every signature; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} not built: run the package build (tk_gb300.build.build())")
    lib = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != TK_OK:
        msg = load().tk_last_error().decode(errors="replace")
        raise TkError(status, msg)


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def i32ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def i64ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def u64ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def i8ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int8))
