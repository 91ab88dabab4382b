"""ctypes binding of libgbs.so (the C ABI in include/gbs.h).

Loading fails loudly: there is no CPU fallback.  Build the library with
``python -m gemmbitserial_gb300.build`` (``__graft_entry__.build()`` does it).
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

GBS_OK, GBS_EINVAL, GBS_ENOMEM, GBS_ECUDA, GBS_ESTATE, GBS_ETIMEOUT, GBS_EUNSUPPORTED = range(7)
GBS_I8, GBS_U8, GBS_I16, GBS_I32, GBS_F32 = range(5)
GBS_LHS, GBS_RHS = 0, 1
GBS_PIPE_AUTO, GBS_PIPE_POPC, GBS_PIPE_BMMA, GBS_PIPE_TC, GBS_PIPE_TC_PAIRS, GBS_PIPE_TC_SMEM = 0, 1, 2, 3, 4, 5
GBS_HOST_IMPORT_AUTO, GBS_HOST_IMPORT_STAGED = 0, 1

# Every entry point include/gbs.h declares, with (restype, argtypes).
u64, i32, vp = C.c_uint64, C.c_int, C.c_void_p


class MatrixInfo(C.Structure):
    _fields_ = [("nbits", u64), ("nrows", u64), ("ncols", u64), ("nrows_a", u64), ("ncols_a", u64),
                ("issigned", i32), ("isbipolar", i32), ("data", vp)]


class CtxInfo(C.Structure):
    _fields_ = [("lhs", MatrixInfo), ("rhs", MatrixInfo), ("lhsBlock", u64), ("rhsBlock", u64),
                ("res", vp), ("pipe", i32)]


SIGNATURES = {
    "gbs_ctx_alloc": (i32, [u64, u64, u64, u64, u64, i32, i32, C.POINTER(vp)]),
    "gbs_ctx_allocate": (i32, [u64, u64, u64, u64, u64, i32, i32, C.POINTER(vp)]),
    "gbs_ctx_dims": (i32, [u64, u64, u64, C.POINTER(u64)]),
    "gbs_matrix_alloc": (i32, [u64, u64, u64, i32, u64, u64, C.POINTER(vp)]),
    "gbs_ctx_free": (i32, [vp]),
    "gbs_ctx_get_info": (i32, [vp, C.POINTER(CtxInfo)]),
    "gbs_import": (i32, [vp, i32, vp, i32, i32, vp]),
    "gbs_import_quantize": (i32, [vp, i32, vp, vp, i32, i32, i32, vp]),
    "gbs_get_bit": (i32, [vp, i32, u64, u64, u64, C.POINTER(i32)]),
    "gbs_set_bit": (i32, [vp, i32, u64, u64, u64, i32]),
    "gbs_get_word": (i32, [vp, i32, u64, u64, u64, C.POINTER(u64)]),
    "gbs_set_word": (i32, [vp, i32, u64, u64, u64, u64]),
    "gbs_clear": (i32, [vp, i32, vp]),
    "gbs_gemm": (i32, [vp, vp]),
    "gbs_gemm_to": (i32, [vp, vp, vp]),
    "gbs_get_result": (i32, [vp, vp, vp]),
    "gbs_sum_rows": (i32, [vp, i32, vp, vp]),
    "gbs_export": (i32, [vp, i32, vp, vp]),
    "gbs_get_planes": (i32, [vp, i32, vp, vp]),
    "gbs_set_pipe": (i32, [vp, i32]),
    "gbs_set_host_import": (i32, [vp, i32]),
    "gbs_set_variant": (i32, [vp, i32]),
    "gbs_gemm_noalloc": (i32, [vp, i32, vp, i32, u64, u64, u64, u64, u64, i32, i32, vp, vp]),
    "gbs_noalloc_scratch_bytes": (u64, []),
    "gbs_adjoint": (i32, [vp, vp, vp, vp, vp]),
    "gbs_fma_peak": (i32, [C.POINTER(C.c_double)]),
    "gbs_tc_peaks": (i32, [C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gbs_group_create": (i32, [C.POINTER(vp), i32, C.POINTER(vp)]),
    "gbs_group_import": (i32, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(i32), vp]),
    "gbs_group_gemm": (i32, [vp, vp]),
    "gbs_group_capture": (i32, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(i32), vp]),
    "gbs_group_replay": (i32, [vp, vp]),
    "gbs_group_status": (i32, [vp, vp]),
    "gbs_group_stats": (i32, [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
    "gbs_group_split": (i32, [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]),
    "gbs_group_free": (i32, [vp]),
    "gbs_debug_group_poison_tile": (i32, [vp, C.c_uint32]),
    "gbs_debug_group_tc_kernel": (i32, [vp]),
    "gbs_pipe_peaks": (i32, [C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gbs_tune": (i32, [vp, i32, C.POINTER(i32), vp]),
    "gbs_tuner_save": (i32, [C.c_char_p]),
    "gbs_tuner_load": (i32, [C.c_char_p, i32]),
    "gbs_tuner_entries": (i32, []),
    "gbs_tuner_clear": (i32, []),
    "gbs_tuner_lookup": (i32, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(C.c_double)]),
    "gbs_last_error": (C.c_char_p, []),
    "gbs_version": (C.c_char_p, []),
    "gbs_debug_fail_alloc_after": (None, [i32]),
    "gbs_debug_launch_count": (u64, []),
    "gbs_debug_last_pair": (i32, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
    "gbs_debug_tc_timeout": (i32, [vp, C.c_uint32, vp]),
    "gbs_debug_tc_error": (C.c_uint32, []),
}

_lib = None


class GBSError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbs error {code}: {msg}")
        self.code = code


def lib_path() -> str:
    return _build.LIB


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"libgbs.so not built ({path}); run python -m gemmbitserial_gb300.build")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != GBS_OK:
        raise GBSError(code, load().gbs_last_error().decode())
