"""ctypes binding of libhssgpu.so (the C ABI declared in include/hssgpu.h).

The library is built in-tree (``hssc_directsolver_gb300/libhssgpu.so``) by
``hssc_directsolver_gb300/build.py``.  There is no CPU fallback: when the
library is missing, :func:`lib` raises, and when no GPU is present every
compute entry point returns ``HSS_ERR_CUDA`` which :func:`check` turns into
an exception.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhssgpu.so")

HSS_OK = 0
HSS_ERR_ARG = 1
HSS_ERR_CUDA = 2
HSS_ERR_SINGULAR = 3
HSS_ERR_NONFINITE = 4
HSS_ERR_RANK = 5
HSS_ERR_STATE = 6
HSS_ERR_NOMEM = 7
ERR_NAMES = {0: "HSS_OK", 1: "HSS_ERR_ARG", 2: "HSS_ERR_CUDA", 3: "HSS_ERR_SINGULAR",
             4: "HSS_ERR_NONFINITE", 5: "HSS_ERR_RANK", 6: "HSS_ERR_STATE", 7: "HSS_ERR_NOMEM"}

HSS_SL_L_2D = 0
HSS_DL_L_2D = 1
HSS_SL_H_2D = 2
HSS_MOD_GAUSS = 0
HSS_MOD_BUMP = 1
HSS_MOD_SQRT_BUMP = 2
HSS_MOD_GAUSS0 = 3
HSS_ID_STEP_TEST = 256
HSS_SKEL_BDRY = 0
HSS_SKEL_RAND = 1
HSS_SKEL_ID = 2
HSS_SKEL_WDEC = 3
HSS_PROXY_BDRY = 0
HSS_PROXY_RAND = 1
HSS_PROXY_WDEC = 2
HSS_PREC_FP64 = 0
HSS_PREC_MIXED = 1
HSS_PREC_DFLOAT = 2
HSS_PREC_DFLOAT_INV = 3
HSS_PREC_TC = 4
HSS_INTER_DENSE = 0
HSS_INTER_LOWRANK = 1


class hss_kernel_params(C.Structure):
    _fields_ = [("flag", C.c_int32), ("pad_", C.c_int32), ("h", C.c_double),
                ("b_alpha", C.c_double), ("b_x0", C.c_double), ("b_y0", C.c_double), ("b_isig", C.c_double),
                ("c_alpha", C.c_double), ("c_x0", C.c_double), ("c_y0", C.c_double), ("c_isig", C.c_double),
                ("kh", C.c_double), ("dr_re", C.c_double), ("dr_im", C.c_double),
                ("b_kind", C.c_int32), ("c_kind", C.c_int32)]


class hss2d_params(C.Structure):
    _fields_ = [("Ng", C.c_int32), ("npan", C.c_int32), ("layers", C.c_int32), ("interform", C.c_int32),
                ("transinv", C.c_int32), ("sym", C.c_int32), ("precision", C.c_int32), ("pad_", C.c_int32),
                ("acc", C.c_double), ("kp", hss_kernel_params), ("k_cut", C.c_int32), ("pad2_", C.c_int32),
                ("seed", C.c_uint64), ("proxy_rule", C.c_int32), ("pad3_", C.c_int32), ("lambda", C.c_double),
                ("skel_rule", C.c_int32), ("pad4_", C.c_int32)]


class HSSError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


_P = C.c_void_p
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "hss_last_error": (C.c_char_p, []),
    "hss_version": (C.c_int, []),
    "hss_device_count": (C.c_int, [_I32P]),
    "hss1d_compress": (C.c_int, [C.POINTER(_P), _P, C.c_int64, C.c_int64, C.c_int32, C.c_double,
                                 C.POINTER(hss_kernel_params), C.c_uint64]),
    "hss_kernel_eval": (C.c_int, [C.POINTER(hss_kernel_params), _DP, C.c_int64, _DP, C.c_int64, _DP]),
    "hss_kernel_eval_device": (C.c_int, [C.POINTER(hss_kernel_params), _P, C.c_int64, _P, C.c_int64, _P, _P]),
    "hss_dr_corrections": (C.c_int, [C.c_double, C.c_double, C.c_double, _DP]),
    "hss_dr_stencil": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_int64, C.c_int32, _I32P, _I64P, _DP,
                                 _I32P]),
    "hss1d_compress_fsym": (C.c_int, [C.POINTER(_P), _P, C.c_int64, C.c_int64, C.c_int32, C.c_double,
                                      C.POINTER(hss_kernel_params), C.c_uint64]),
    "hss1d_compress_batch_ex": (C.c_int, [C.POINTER(_P), C.c_int32, _I64P, C.POINTER(C.c_void_p), _I64P, C.c_int32,
                                          C.c_double, C.POINTER(hss_kernel_params), C.POINTER(C.c_uint64), _P,
                                          C.c_int32]),
    "hss1d_compress_batch": (C.c_int, [C.POINTER(_P), C.c_int32, _I64P, C.POINTER(C.c_void_p), _I64P, C.c_int32,
                                       C.c_double, C.POINTER(hss_kernel_params), C.POINTER(C.c_uint64)]),
    "hss1d_compress_rect": (C.c_int, [C.POINTER(_P), _P, C.c_int64, C.c_int64, _P, C.c_int64, C.c_int64,
                                      C.c_int32, C.c_double, C.POINTER(hss_kernel_params), C.c_uint64]),
    "hss1d_rect_info": (C.c_int, [_P, _I64P, _I32P, _I32P, _I32P, _I32P]),
    "hss1d_sum": (C.c_int, [_P, _P, C.c_double, C.POINTER(_P)]),
    "hss1d_compress_lr": (C.c_int, [C.POINTER(_P), _P, _P, C.c_int64, C.c_int32, C.c_int64, C.c_int64, C.c_int32,
                                    C.c_double, C.c_uint64]),
    "hss1d_forest_info": (C.c_int, [_P, _I32P, _I64P, _I32P, _I64P]),
    "hss1d_is_complex": (C.c_int, [_P, _I32P]),
    "hss2d_is_complex": (C.c_int, [_P, _I32P]),
    "hss1d_recompress": (C.c_int, [_P, C.c_double, C.POINTER(_P)]),
    "hss1d_info": (C.c_int, [_P, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P, _I32P]),
    "hss1d_export_box": (C.c_int, [_P, C.c_int32, _I32P, _I32P, _I32P, _I32P, _DP, _DP]),
    "hss1d_invert": (C.c_int, [_P]),
    "hss1d_transforminv": (C.c_int, [_P, C.POINTER(_P)]),
    "hss1d_apply": (C.c_int, [_P, _P, _P, C.c_int32]),
    "hss1d_applyinv": (C.c_int, [_P, _P, _P, C.c_int32]),
    "hss1d_applyinv_device": (C.c_int, [_P, _P, _P, C.c_int32, _P]),
    "hss1d_solve": (C.c_int, [_P, _P, _P, C.c_int32, C.c_double, C.c_int32, _DP, _I32P]),
    "hss1d_solve_device": (C.c_int, [_P, _P, _P, C.c_int32, C.c_double, C.c_int32, _DP, _I32P, _P]),
    "hss1d_set_precision": (C.c_int, [_P, C.c_int32]),
    "hss1d_transpose": (C.c_int, [_P, C.POINTER(_P)]),
    "hss2d_set_autotune": (C.c_int, [_P, C.c_int32]),
    "hss1d_scalarmult": (C.c_int, [_P, C.c_double]),
    "hss1d_dense_matrix": (C.c_int, [_P, C.c_int32, _P]),
    "hss1d_apply_submatrix": (C.c_int, [_P, _P, _P, _P, C.c_int32, _P]),
    "hss1d_apply_submatrix_boxes": (C.c_int, [_P, _P, _P, _P, _P]),
    "hss1d_destroy": (C.c_int, [_P]),
    "hss_mlp_create": (C.c_int, [C.POINTER(_P), C.c_int32, C.c_int32, C.c_uint64]),
    "hss_mlp_nparams": (C.c_int, [_P, _I32P]),
    "hss_mlp_get_params": (C.c_int, [_P, _P]),
    "hss_mlp_set_params": (C.c_int, [_P, _P]),
    "hss_mlp_grad": (C.c_int, [_P, _P, _P, C.c_int32, _P, C.POINTER(C.c_float)]),
    "hss_mlp_train": (C.c_int, [_P, _P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.POINTER(C.c_float)]),
    "hss_mlp_predict": (C.c_int, [_P, _P, C.c_int32, _P]),
    "hss_mlp_destroy": (C.c_int, [_P]),
    "hss1d_features": (C.c_int, [_P, _P, _P]),
    "hss1d_id_stats": (C.c_int, [_P, _I64P, _I64P, _I32P]),
    "hss1d_phase_times": (C.c_int, [_P, _DP]),
    "hss1d_compress_batch_learned": (C.c_int, [C.POINTER(_P), C.c_int32, _I64P, C.POINTER(C.c_void_p), _I64P,
                                               C.c_int32, C.c_double, _P, _P, _P]),
    "hss2d_build_tree": (C.c_int, [C.POINTER(_P), C.POINTER(hss2d_params)]),
    "hss2d_compress": (C.c_int, [_P]),
    "hss2d_invert": (C.c_int, [_P]),
    "hss2d_apply": (C.c_int, [_P, _P, _P, C.c_int32]),
    "hss2d_apply_device": (C.c_int, [_P, _P, _P, C.c_int32, _P]),
    "hss2d_applyinv": (C.c_int, [_P, _P, _P, C.c_int32]),
    "hss2d_applyinv_device": (C.c_int, [_P, _P, _P, C.c_int32, _P]),
    "hss2d_solve": (C.c_int, [_P, _P, _P, C.c_int32, C.c_double, C.c_int32, _DP, _I32P]),
    "hss2d_solve_device": (C.c_int, [_P, _P, _P, C.c_int32, C.c_double, C.c_int32, _DP, _I32P, _P]),
    "hss2d_info": (C.c_int, [_P, _I32P, _I32P, _I64P]),
    "hss2d_box_sizes": (C.c_int, [_P, _I32P, _I32P, _I32P]),
    "hss2d_export_box": (C.c_int, [_P, C.c_int32, _I32P, _I32P, _DP, _DP]),
    "hss2d_export_inverse": (C.c_int, [_P, C.c_int32, _DP, _DP]),
    "hss2d_interp_ranks": (C.c_int, [_P, _I32P, _I32P]),
    "hss2d_phase_times": (C.c_int, [_P, _DP]),
    "hss2d_bicgstab": (C.c_int, [_P, _P, _P, _P, C.c_int32, C.c_double, C.c_int32, _DP, _I32P]),
    "hss2d_gmres": (C.c_int, [_P, _P, _P, _P, C.c_int32, C.c_double, C.c_int32, C.c_int32, _DP, _I32P]),
    "hss2d_kernel_residual_rows": (C.c_int, [_P, C.c_int64, C.c_int64, _P, _P, C.c_int32, _P]),
    "hss2d_proxy_points": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _DP, C.c_int32, _I32P]),
    "hss2d_solve_bytes": (C.c_int, [_P, _I64P]),
    "hss2d_solve_launches": (C.c_int, [_P, C.c_int32, _I32P]),
    "hss2d_destroy": (C.c_int, [_P]),
    "hss_batched_inverse_device": (C.c_int, [_P, C.c_int32, C.c_int32, _P, _P]),
    "hss_batched_inverse_device_f32": (C.c_int, [_P, C.c_int32, C.c_int32, _P, _P]),
    "hss_batched_inverse_noalloc_device": (C.c_int, [_P, C.c_int32, C.c_int32, _P, _P]),
    "hss_batched_lstsq_device": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "hss_batched_lstsq_device_ex": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "hss_batched_id_device": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_uint64,
                                        C.c_int32, _P, _P, _P, _P]),
    "hss_batched_gemm_device": (C.c_int, [_P, _P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "hss_batched_gemv_tc_device": (C.c_int, [_P, _P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "hss2d_kernel_residual": (C.c_int, [_P, _P, _P, C.c_int32, _P]),
    "hss1d_kernel_residual": (C.c_int, [_P, _P, _P, C.c_int32, _P]),
}

_lib = None
_lock = threading.Lock()


def lib() -> C.CDLL:
    """Load libhssgpu.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing: run hssc_directsolver_gb300/build.py "
                                  "(the CUDA library is required; there is no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(code: int) -> None:
    if code != HSS_OK:
        msg = lib().hss_last_error()
        raise HSSError(code, msg.decode() if msg else "")


def device_count() -> int:
    n = C.c_int32(0)
    check(lib().hss_device_count(C.byref(n)))
    return n.value


def ptr(a) -> C.c_void_p:
    """Raw data pointer of a contiguous numpy array or torch tensor."""
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a.ctypes.data)
