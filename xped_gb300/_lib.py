"""ctypes bindings of the native library (include/xgb.h, include/xgb_tensor.h).

The library is built in-tree by ``xped_gb300.build.build()``; importing this
module without it raises, there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libxgb.so"

MAX_LEGS = 8


class PermTask(C.Structure):
    _fields_ = [("dst_base", C.c_int64), ("nelem", C.c_int64), ("rank", C.c_int32), ("n_contrib", C.c_int32),
                ("contrib0", C.c_int32), ("pad", C.c_int32), ("dims", C.c_int32 * MAX_LEGS),
                ("dst_stride", C.c_int64 * MAX_LEGS)]


class PermContrib(C.Structure):
    _fields_ = [("src_base", C.c_int64), ("coeff", C.c_double), ("src_stride", C.c_int64 * MAX_LEGS)]


class GemmDesc(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("k", C.c_int64), ("a_off", C.c_int64), ("lda", C.c_int64),
                ("b_off", C.c_int64), ("ldb", C.c_int64), ("c_off", C.c_int64), ("ldc", C.c_int64),
                ("trans_a", C.c_int32), ("trans_b", C.c_int32)]


class SvdDesc(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("a_off", C.c_int64), ("u_off", C.c_int64),
                ("s_off", C.c_int64), ("vt_off", C.c_int64)]


class QrDesc(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("a_off", C.c_int64), ("q_off", C.c_int64),
                ("q_cols", C.c_int64), ("r_off", C.c_int64), ("r_rows", C.c_int64)]


class Copy2dDesc(C.Structure):
    _fields_ = [("src_off", C.c_int64), ("src_ld", C.c_int64), ("dst_off", C.c_int64), ("dst_ld", C.c_int64),
                ("rows", C.c_int64), ("cols", C.c_int64)]


P = C.c_void_p
i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
dblp = C.POINTER(C.c_double)
fltp = C.POINTER(C.c_float)

# (name, restype, argtypes)
PROTOS = [
    # runtime / kernel level
    ("xgb_init", C.c_int, [C.c_int]),
    ("xgb_shutdown", C.c_int, []),
    ("xgb_last_error", C.c_char_p, []),
    ("xgb_synchronize", C.c_int, []),
    ("xgb_malloc", C.c_int, [C.POINTER(P), C.c_size_t]),
    ("xgb_free", C.c_int, [P]),
    ("xgb_memcpy_h2d", C.c_int, [P, P, C.c_size_t]),
    ("xgb_memcpy_d2h", C.c_int, [P, P, C.c_size_t]),
    ("xgb_memset_zero", C.c_int, [P, C.c_size_t]),
    ("xgb_launch_count", C.c_int64, []),
    ("xgb_grouped_gemm", C.c_int, [C.c_int, C.c_int, C.POINTER(GemmDesc), P, P, P, C.c_double, C.c_double, P]),
    ("xgb_permute", C.c_int, [C.c_int, C.POINTER(PermTask), C.c_int, C.POINTER(PermContrib), P, P, P]),
    ("xgb_svd_workspace_bytes", C.c_size_t, [C.c_int, C.POINTER(SvdDesc)]),
    ("xgb_batched_svd", C.c_int, [C.c_int, C.POINTER(SvdDesc), P, P, P, P, P, P]),
    ("xgb_truncate", C.c_int, [C.c_int, i64p, i32p, P, C.c_int64, C.c_double, C.c_int, P, P, P]),
    ("xgb_qr_workspace_bytes", C.c_size_t, [C.c_int, C.POINTER(QrDesc)]),
    ("xgb_batched_qr", C.c_int, [C.c_int, C.POINTER(QrDesc), P, P, P, P, P]),
    ("xgb_absmax", C.c_int, [P, C.c_int64, P, P]),
    ("xgb_scale_by_inv_absmax", C.c_int, [P, C.c_int64, P, P]),
    ("xgb_scale", C.c_int, [P, C.c_int64, C.c_double, P]),
    ("xgb_copy2d_batched", C.c_int, [C.c_int, C.POINTER(Copy2dDesc), P, P, P]),
    ("xgb_diag_from_vec", C.c_int, [C.c_int, C.POINTER(Copy2dDesc), C.c_int, P, P, P]),
    ("xgb_diag_apply", C.c_int, [C.c_int, C.POINTER(Copy2dDesc), C.c_int, P, P]),
    # tensor level
    ("xgb_basis_create", P, [C.c_int, C.c_int, i32p, i64p, C.c_int]),
    ("xgb_basis_conj", P, [P]),
    ("xgb_basis_combine", P, [P, P]),
    ("xgb_basis_forget_history", P, [P]),
    ("xgb_basis_info", C.c_int, [P, i32p, i64p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("xgb_basis_trees", C.c_int, [P, C.c_int, i64p, C.c_int]),
    ("xgb_basis_release", None, [P]),
    ("xgb_tensor_zeros", P, [C.c_int, C.POINTER(P), C.c_int, C.POINTER(P)]),
    ("xgb_tensor_identity", P, [C.c_int, C.POINTER(P), C.c_int, C.POINTER(P)]),
    ("xgb_tensor_meta", P, [C.c_int, C.POINTER(P), C.c_int, C.POINTER(P)]),
    ("xgb_tensor_sectors", C.c_int, [P, i32p, i64p, i64p]),
    ("xgb_tensor_size", C.c_int64, [P]),
    ("xgb_tensor_rank", C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("xgb_tensor_leg", P, [P, C.c_int]),
    ("xgb_tensor_coupled", P, [P, C.c_int]),
    ("xgb_tensor_upload", C.c_int, [P, dblp, C.c_int64]),
    ("xgb_tensor_download", C.c_int, [P, dblp, C.c_int64]),
    ("xgb_tensor_device_data", P, [P]),
    ("xgb_tensor_permute", P, [P, C.c_int, i32p, C.c_int]),
    ("xgb_tensor_permute_adj", P, [P, C.c_int, i32p, C.c_int]),
    ("xgb_tensor_matmul_backward", C.c_int, [P, P, P, C.POINTER(P), C.POINTER(P)]),
    ("xgb_tensor_svd_backward", P, [P, P, P, P, P, P, P]),
    ("xgb_tensor_twist", P, [P, C.c_int]),
    ("xgb_tensor_adjoint", P, [P]),
    ("xgb_tensor_matmul", P, [P, P, C.c_int, C.c_int]),
    ("xgb_tensor_contract", P, [P, P, i32p, C.c_int, i32p, C.c_int, C.c_int]),
    ("xgb_tensor_scale", P, [P, C.c_double]),
    ("xgb_tensor_max_norm", C.c_double, [P]),
    ("xgb_tensor_normalize_max", P, [P]),
    ("xgb_tensor_tsvd", C.c_int, [P, C.c_int64, C.c_double, C.c_int, C.POINTER(P), C.POINTER(P), C.POINTER(P),
                                  dblp, dblp, i32p]),
    ("xgb_tensor_tsvd_randomized", C.c_int, [P, C.c_int64, C.c_double, C.c_int, i64p, C.c_int, C.c_uint64, P,
                                             C.c_double, C.POINTER(P), C.POINTER(P), C.POINTER(P), dblp, dblp, i32p,
                                             i64p, i32p]),
    ("xgb_tensor_tqr", C.c_int, [P, C.POINTER(P), C.POINTER(P)]),
    ("xgb_decompose", C.c_int, [P, P, C.c_int64, C.POINTER(P), C.POINTER(P)]),
    ("xgb_tensor_release", None, [P]),
    ("xgb_ctm_create", P, [P, C.c_int64]),
    ("xgb_ctm_init", C.c_int, [P]),
    ("xgb_ctm_grow_all", C.c_int, [P]),
    ("xgb_ctm_set_svd", C.c_int, [P, C.c_int, C.c_int, C.c_uint64, C.c_int64, C.c_double]),
    ("xgb_ctm_stats", C.c_int, [P, i64p]),
    ("xgb_ctm_set_warm_start", C.c_int, [P, C.c_int]),
    ("xgb_ctm_set_sketch_unseen", C.c_int, [P, C.c_int]),
    ("xgb_ctm_set_concurrent", C.c_int, [P, C.c_int]),
    ("xgb_ctm_set_sketch_precision", C.c_int, [P, C.c_int]),
    ("xgb_ctm_set_residual_tol", C.c_int, [P, C.c_double]),
    ("xgb_ctm_residual_stats", C.c_int, [P, i64p, dblp]),
    ("xgb_ctm_set_gemm_precision", C.c_int, [P, C.c_int]),
    ("xgb_set_gemm_precision", C.c_int, [C.c_int]),
    ("xgb_ctm_record", C.c_int, [P, C.c_int]),
    ("xgb_ctm_record_count", C.c_int, [P]),
    ("xgb_ctm_record_get", C.c_int, [P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), i64p, i32p,
                                     C.POINTER(C.c_float), i64p, i64p, i64p, dblp, i64p]),
    ("xgb_ctm_rdm", P, [P, C.c_int]),
    ("xgb_tensor_svspec", C.c_int, [P, i32p, i64p, dblp, C.c_int64]),
    ("xgb_ctm_solve", C.c_int, [P, P, C.c_double, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_int]),
    ("xgb_rank_model_num_params", C.c_int, []),
    ("xgb_rank_model_num_features", C.c_int, []),
    ("xgb_rank_model_create", P, [C.c_uint64]),
    ("xgb_rank_model_release", None, [P]),
    ("xgb_rank_model_get_params", C.c_int, [P, fltp, C.c_int]),
    ("xgb_rank_model_set_params", C.c_int, [P, fltp, C.c_int]),
    ("xgb_rank_model_predict", C.c_int, [P, fltp, C.c_int64, fltp]),
    ("xgb_rank_model_gradient", C.c_int, [P, fltp, fltp, C.c_int64, fltp, dblp]),
    ("xgb_rank_model_train", C.c_int, [P, fltp, fltp, C.c_int64, C.c_int, C.c_float, dblp]),
    ("xgb_ctm_set_rank_model", C.c_int, [P, P, C.c_double, C.c_int64, C.c_int, C.c_uint64]),
    ("xgb_tensor_bond_expectation", C.c_int, [P, P, dblp]),
    ("xgb_ctm_move", C.c_int, [P, C.c_char]),
    ("xgb_ctm_get", P, [P, C.c_int]),
    ("xgb_ctm_set", C.c_int, [P, C.c_int, P]),
    ("xgb_ctm_release", None, [P]),
    ("xgb_tensor_serialize", C.c_int, [P, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    ("xgb_tensor_deserialize", P, [C.c_void_p, C.c_int64]),
    ("xgb_ctm_serialize", C.c_int, [P, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    ("xgb_ctm_deserialize", P, [P, C.c_void_p, C.c_int64]),
    ("xgb_su_create", P, [C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(P), C.c_int64]),
    ("xgb_su_step", C.c_int, [P, P, P]),
    ("xgb_su_step_h", C.c_int, [P, C.c_int, C.c_int, P]),
    ("xgb_su_step_v", C.c_int, [P, C.c_int, C.c_int, P]),
    ("xgb_su_get", P, [P, C.c_int, C.c_int]),
    ("xgb_su_release", None, [P]),
    ("xgb_permute_plan_host", C.c_int, [P, C.c_int, i32p, C.c_int, C.c_uint32, C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.POINTER(PermTask), C.c_int, C.POINTER(PermContrib),
                                        C.c_int, C.POINTER(P)]),
    ("xgb_gemm_plan_host", C.c_int, [P, C.c_int, P, C.c_int, C.POINTER(C.c_int), C.POINTER(GemmDesc), C.c_int,
                                     C.POINTER(P)]),
    ("xgb_contract_perms", C.c_int, [i32p, C.c_int, C.c_int, i32p, C.c_int, C.c_int, C.c_int, i32p]),
    ("xgb_plan_cache_stats", C.c_int, [i64p]),
]

_lib = None


class XgbError(RuntimeError):
    pass


def lib():
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"native library {LIB_PATH} is missing: run xped_gb300.build.build() first")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in PROTOS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    msg = lib().xgb_last_error()
    return msg.decode() if msg else ""


def check(rc, what="xgb call"):
    if isinstance(rc, int) and rc < 0:
        raise XgbError(f"{what} failed ({rc}): {last_error()}")
    return rc


def check_handle(h, what="xgb call"):
    if not h:
        raise XgbError(f"{what} failed: {last_error()}")
    return h


_initialised = False


def ensure_device(device: int = 0):
    """Initialise the CUDA runtime of the library (once)."""
    global _initialised
    if not _initialised:
        check(lib().xgb_init(device), "xgb_init")
        _initialised = True


PROTOS_EXTRA = [
    ("xgb_stream_handle", C.c_void_p, []),
    ("xgb_gemm_tc_status", C.c_int, []),
    ("xgb_profile_enable", C.c_int, [C.c_int]),
    ("xgb_profile_reset", C.c_int, []),
    ("xgb_profile_read", C.c_int, [C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("xgb_event_record", C.c_int, [C.c_int]),
    ("xgb_event_elapsed_ms", C.c_double, [C.c_int, C.c_int]),
    ("xgb_svd_last_sweeps", C.c_int, [i32p, C.c_int]),
    ("xgb_batched_svd_noalloc", C.c_int, [C.c_int, C.POINTER(SvdDesc), P, P, P, P, P]),
    ("xgb_batched_svd_noalloc_capacity_bytes", C.c_size_t, []),
    ("xgb_autotune_set", C.c_int, [C.c_int]),
    ("xgb_autotune_reset", C.c_int, []),
    ("xgb_autotune_stats", C.c_int, [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    ("xgb_autotune_candidates", C.c_int, [i32p, i32p, C.c_int]),
    ("xgb_autotune_choices", C.c_int, [i32p, i32p, C.c_int]),
    ("xgb_autotune_gemm", C.c_int, [C.c_int, C.POINTER(GemmDesc), P, P, C.POINTER(C.c_double), i32p]),
    ("xgb_grouped_gemm_f64_config", C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(GemmDesc), P, P, P, C.c_double,
                                              C.c_double, P]),
    ("xgb_autotune_save", C.c_int, [C.c_char_p]),
    ("xgb_autotune_load", C.c_int, [C.c_char_p]),
]
PROTOS.extend(PROTOS_EXTRA)

KERNEL_KINDS = ["gemm_f64", "permute", "svd_jacobi", "truncate", "qr", "absmax", "scale", "copy2d", "diag", "gemm_tc", "sketch", "mlp", "gemm_f32", "gemm_f64tc"]


def profile_read():
    """{kind: (launches, device ms, algorithmic work)} for every kernel kind."""
    out = {}
    for k, name in enumerate(KERNEL_KINDS):
        n, ms, w = C.c_int64(), C.c_double(), C.c_double()
        check(lib().xgb_profile_read(k, C.byref(n), C.byref(ms), C.byref(w)), "profile_read")
        out[name] = (n.value, ms.value, w.value)
    return out
