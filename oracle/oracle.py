"""Python access to the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It is the oracle the GPU path is compared
against, never part of the product path.

* ``liboracle.so`` (built from ``gbs_oracle.c``) restates the reference's
  generic algorithm in C; every routine there cites the reference file:line.
* ``libgbsref.so`` is the unmodified reference compiled from its own header by
  ``make -C oracle ref``; it exists only where the reference sources exist.
* ``adjoint_fp64`` is the float64 statement of the adjoint (no reference
  counterpart exists for it).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libgbsref.so")

DT_I8, DT_U8, DT_I16, DT_I32 = 0, 1, 2, 3
_NP2DT = {np.dtype(np.int8): DT_I8, np.dtype(np.uint8): DT_U8,
          np.dtype(np.int16): DT_I16, np.dtype(np.int32): DT_I32, np.dtype(np.float32): 4}

_lib = None
_ref = None

u64 = C.c_uint64
vp = C.c_void_p


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference driver when ``ref`` and its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:  # the Makefile knows where the reference lies (REFDIR)
        subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        L.orc_ctx_alloc.restype = vp
        L.orc_ctx_alloc.argtypes = [u64, u64, u64, u64, u64, C.c_int, C.c_int]
        L.orc_ctx_free.argtypes = [vp]
        L.orc_ctx_dims.argtypes = [vp, vp]
        L.orc_planes.restype = C.POINTER(C.c_uint64)
        L.orc_planes.argtypes = [vp, C.c_int]
        L.orc_res.restype = C.POINTER(C.c_int32)
        L.orc_res.argtypes = [vp]
        L.orc_import.argtypes = [vp, C.c_int, vp, C.c_int, C.c_int]
        L.orc_export.argtypes = [vp, C.c_int, vp]
        L.orc_import_quantize.argtypes = [vp, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int]
        L.orc_sum_rows.argtypes = [vp, C.c_int, vp]
        L.orc_gemm.argtypes = [vp]
        L.orc_gemm_threads.argtypes = [vp, C.c_int]
        L.orc_naive_gemm.argtypes = [vp, vp, vp, u64, u64, u64]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_SO)
        R.ref_run.argtypes = [u64, u64, u64, u64, u64, C.c_int, C.c_int,
                              vp, C.c_int, C.c_int, vp, C.c_int, C.c_int, vp, vp, vp]
        R.ref_sum_rows.argtypes = [u64, u64, u64, C.c_int, vp, C.c_int, vp]
        R.ref_roundtrip.argtypes = [u64, u64, u64, C.c_int, vp, C.c_int, vp]
        R.ref_quantize_export.argtypes = [u64, u64, u64, vp, vp, C.c_int, C.c_int, C.c_int, vp]
        R.ref_time_gemm.restype = C.c_double
        R.ref_time_gemm.argtypes = [u64, u64, u64, u64, u64, C.c_int, C.c_int,
                                    vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp]
        _ref = R
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(vp)


class OracleContext:
    """An oracle GEMM context: the C restatement of GEMMContext (gemmbitserial.hpp:379-452)."""

    def __init__(self, M, K, N, wA, wB, sA, sB):
        self.M, self.K, self.N, self.wA, self.wB = int(M), int(K), int(N), int(wA), int(wB)
        self.h = lib().orc_ctx_alloc(M, K, N, wA, wB, int(bool(sA)), int(bool(sB)))
        d = np.zeros(6, np.uint64)
        lib().orc_ctx_dims(self.h, _ptr(d))
        self.dims = [int(x) for x in d]

    def import_(self, side: int, arr: np.ndarray, colmajor: bool = False):
        arr = np.ascontiguousarray(arr)
        lib().orc_import(self.h, side, _ptr(arr), _NP2DT[arr.dtype], int(colmajor))

    def import_quantize(self, side: int, arr: np.ndarray, thresholds: np.ndarray, colmajor: bool = False):
        """importRegularAndQuantize (gemmbitserial.hpp:282-305); thresholds shaped [nThres][nrows]."""
        arr = np.ascontiguousarray(arr)
        thr = np.ascontiguousarray(thresholds, dtype=arr.dtype)
        nthres = int(thr.shape[0]) if thr.ndim == 2 else 0
        rc = lib().orc_import_quantize(self.h, side, _ptr(arr), _ptr(thr) if thr.size else None, nthres,
                                       _NP2DT[arr.dtype], int(colmajor))
        if rc != 0:
            raise ValueError("threshold quantization needs an unsigned matrix")

    def gemm(self, threads: int = 1):
        if threads > 1:
            lib().orc_gemm_threads(self.h, threads)
        else:
            lib().orc_gemm(self.h)

    def res(self) -> np.ndarray:
        n = self.M * self.N
        if n == 0:
            return np.zeros((self.N, self.M), np.int32)
        return np.ctypeslib.as_array(lib().orc_res(self.h), shape=(n,)).copy().reshape(self.N, self.M)

    def planes(self, side: int) -> np.ndarray:
        rows_a = self.dims[side]
        wpr = self.dims[2 + side] // 64
        bits = self.wB if side else self.wA
        n = bits * rows_a * wpr
        if n == 0:
            return np.zeros((bits, rows_a, wpr), np.uint64)
        return np.ctypeslib.as_array(lib().orc_planes(self.h, side), shape=(n,)).copy().reshape(bits, rows_a, wpr)

    def sum_rows(self, side: int) -> np.ndarray:
        rows = self.N if side else self.M
        out = np.zeros(rows + 1, np.int32)
        lib().orc_sum_rows(self.h, side, _ptr(out))
        return out[:rows]

    def export(self, side: int) -> np.ndarray:
        rows = self.N if side else self.M
        out = np.zeros(rows * self.K + 1, np.int32)
        lib().orc_export(self.h, side, _ptr(out))
        return out[:rows * self.K].reshape(rows, self.K)

    def close(self):
        if self.h:
            lib().orc_ctx_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


def oracle_gemm(A, B, wA, wB, sA, sB, colmajorA=False, colmajorB=False, threads=1):
    """Full oracle pass; A is M x K (or K x M storage when colmajorA), B is N x K. Returns res[N, M]."""
    if colmajorA:
        M, K = A.shape[1], A.shape[0]
    else:
        M, K = A.shape
    N = B.shape[1] if colmajorB else B.shape[0]
    ctx = OracleContext(M, K, N, wA, wB, sA, sB)
    ctx.import_(0, A, colmajorA)
    ctx.import_(1, B, colmajorB)
    ctx.gemm(threads)
    r = ctx.res()
    ctx.close()
    return r


def ref_gemm(A, B, wA, wB, sA, sB, colmajorA=False, colmajorB=False, want_planes=False):
    """Run the compiled reference. Returns (res[N, M], dims, planes or None)."""
    A = np.ascontiguousarray(A)
    B = np.ascontiguousarray(B)
    M, K = (A.shape[1], A.shape[0]) if colmajorA else A.shape
    N = B.shape[1] if colmajorB else B.shape[0]
    res = np.zeros(max(M * N, 1), np.int32)
    dims = np.zeros(6, np.uint64)
    planes = None
    pp = None
    if want_planes:
        oc = OracleContext(M, K, N, wA, wB, sA, sB)
        na = wA * oc.dims[0] * (oc.dims[2] // 64)
        nb = wB * oc.dims[1] * (oc.dims[3] // 64)
        oc.close()
        planes = np.zeros(na + nb + 1, np.uint64)
        pp = _ptr(planes)
    ref().ref_run(M, K, N, wA, wB, int(bool(sA)), int(bool(sB)),
                  _ptr(A), _NP2DT[A.dtype], int(colmajorA), _ptr(B), _NP2DT[B.dtype], int(colmajorB),
                  _ptr(res), _ptr(dims), pp)
    return res[:M * N].reshape(N, M), [int(x) for x in dims], planes


def naive_gemm(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """test/testhelpers.hpp:34-45 naive_int_gemm: res[n, m] = sum_k A[m,k]*B[n,k] (int32 wrap)."""
    r = A.astype(np.int64) @ B.astype(np.int64).T  # [M, N]
    return (r.T & 0xFFFFFFFF).astype(np.uint32).view(np.int32)


def decode_values(x: np.ndarray, bits: int, signed: bool, raw_u8: bool = False) -> np.ndarray:
    """The integer each element represents after import (the export of gemmbitserial.hpp:313-333)."""
    x = x.astype(np.int64)
    if bits == 1 and signed:
        return np.where((x & 1) if raw_u8 else (x > 0), 1, -1).astype(np.int64)
    q = x & ((1 << bits) - 1)
    if signed:
        q = np.where(q >= (1 << (bits - 1)), q - (1 << bits), q)
    return q


def adjoint_fp64(dC: np.ndarray, Avals: np.ndarray, Bvals: np.ndarray):
    """float64 adjoint of res[n, m] = sum_k A[m,k] B[n,k] given dC[n, m]:
    dA[m, k] = sum_n dC[n, m] B[n, k];  dB[n, k] = sum_m dC[n, m] A[m, k]."""
    d = dC.astype(np.float64)
    dA = d.T @ Bvals.astype(np.float64)
    dB = d @ Avals.astype(np.float64)
    return dA, dB


def quantize_values(arr: np.ndarray, thresholds: np.ndarray, bits: int, colmajor: bool = False) -> np.ndarray:
    """The values an unsigned ``bits``-bit matrix holds after importRegularAndQuantize of ``arr``
    (rows x cols, or cols x rows when ``colmajor``) with thresholds [nThres][rows]."""
    rows, cols = (arr.shape[1], arr.shape[0]) if colmajor else arr.shape
    ctx = OracleContext(rows, cols, 1, bits, 1, False, False)
    ctx.import_quantize(0, arr, thresholds, colmajor)
    out = np.zeros((rows, cols), np.int32)
    if rows * cols:
        lib().orc_export(ctx.h, 0, _ptr(out))
    return out


def ref_quantize_values(arr: np.ndarray, thresholds: np.ndarray, bits: int, colmajor: bool = False) -> np.ndarray:
    """The same through the compiled reference (oracle/_ref)."""
    arr = np.ascontiguousarray(arr)
    thr = np.ascontiguousarray(thresholds, dtype=arr.dtype)
    rows, cols = (arr.shape[1], arr.shape[0]) if colmajor else arr.shape
    out = np.zeros((rows, cols), np.int32)
    nthres = int(thr.shape[0]) if thr.ndim == 2 else 0
    ref().ref_quantize_export(rows, cols, bits, _ptr(arr), _ptr(thr) if thr.size else None, nthres,
                              _NP2DT[arr.dtype], int(colmajor), _ptr(out))
    return out


def import_values(arr: np.ndarray, bits: int, signed: bool, colmajor: bool = False) -> np.ndarray:
    """The values a ``bits``-bit matrix holds after importRegular of ``arr`` (exportRegular of it)."""
    arr = np.ascontiguousarray(arr)
    rows, cols = (arr.shape[1], arr.shape[0]) if colmajor else arr.shape
    ctx = OracleContext(rows, cols, 1, bits, 1, signed, False)
    ctx.import_(0, arr, colmajor)
    out = np.zeros((rows, cols), np.int32)
    if rows * cols:
        lib().orc_export(ctx.h, 0, _ptr(out))
    return out


def ref_import_values(arr: np.ndarray, bits: int, signed: bool) -> np.ndarray:
    """The same through the compiled reference (row-major input)."""
    arr = np.ascontiguousarray(arr)
    rows, cols = arr.shape
    out = np.zeros((rows, cols), np.int32)
    ref().ref_roundtrip(rows, cols, bits, int(bool(signed)), _ptr(arr), _NP2DT[arr.dtype], _ptr(out))
    return out
