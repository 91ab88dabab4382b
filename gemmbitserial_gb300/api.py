"""Python mirror of gemmbitserial's public API over the C ABI.

Same names, argument meaning and error behaviour as the reference's hot path
(gemmbitserial.hpp:379-479, arch-generic.hpp:78-100, 331-345):

    ctx = allocGEMMContext(M, K, N, lhsBits, rhsBits, lhsSigned, rhsSigned)
    ctx.lhs.importRegular(A)          # M x K
    ctx.rhs.importRegular(BT)         # N x K (B transposed)
    gemmBitSerial(ctx)
    res = ctx.res                     # N*M int32, transposed result
    deallocGEMMContext(ctx)

All compute runs in libgbs.so on the GPU.  Inputs may be numpy arrays (host)
or torch CUDA tensors (device).  Integer element types select the reference's
import overload: uint8 is the raw-bit overload (gemmbitserial.hpp:249), the
signed types go through quantize<T> (gemmbitserial.hpp:170).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi

_NP2DT = {np.dtype(np.int8): _capi.GBS_I8, np.dtype(np.uint8): _capi.GBS_U8,
          np.dtype(np.int16): _capi.GBS_I16, np.dtype(np.int32): _capi.GBS_I32}


def _stream_handle(stream):
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return C.c_void_p(torch.cuda.current_stream().cuda_stream)
        except ImportError:
            pass
        return C.c_void_p(0)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def _src(arr, allow_float: bool = False):
    """(pointer, dtype code, keepalive) for a numpy array or torch tensor."""
    try:
        import torch
        if isinstance(arr, torch.Tensor):
            t = arr.contiguous()
            dt = {torch.int8: _capi.GBS_I8, torch.uint8: _capi.GBS_U8, torch.int16: _capi.GBS_I16,
                  torch.int32: _capi.GBS_I32, torch.float32: _capi.GBS_F32}[t.dtype]
            if dt == _capi.GBS_F32 and not allow_float:
                raise TypeError("float input is not accepted here")
            return C.c_void_p(t.data_ptr()), dt, t
    except ImportError:
        pass
    a = np.ascontiguousarray(arr)
    if a.dtype == np.float32 and allow_float:
        return C.c_void_p(a.ctypes.data), _capi.GBS_F32, a
    if a.dtype not in _NP2DT:
        raise TypeError(f"unsupported element type {a.dtype}; use int8, uint8, int16 or int32")
    return C.c_void_p(a.ctypes.data), _NP2DT[a.dtype], a


def _release(keep, source, stream) -> None:
    """Drops a contiguous copy _src made of a device tensor.  The import may still
    read it on `stream`; torch reuses a freed block in the order of the stream it
    was allocated on (the current one), so for another stream wait first."""
    if stream is None or keep is source:
        return
    try:
        import torch
    except ImportError:
        return
    if isinstance(keep, torch.Tensor) and keep.is_cuda:
        torch.cuda.synchronize(keep.device)


class BitSerialMatrix:
    """One operand of a context (gemmbitserial.hpp:19-50); the planes live on the GPU."""

    def __init__(self, ctx: "GEMMContext", side: int):
        self._ctx = ctx
        self._side = side

    def _info(self):
        i = self._ctx._info()
        return i.rhs if self._side else i.lhs

    @property
    def nbits(self): return self._info().nbits

    @property
    def nrows(self): return self._info().nrows

    @property
    def ncols(self): return self._info().ncols

    @property
    def nrows_a(self): return self._info().nrows_a

    @property
    def ncols_a(self): return self._info().ncols_a

    @property
    def issigned(self): return bool(self._info().issigned)

    @property
    def data(self):
        """Device address of the planes, layout [nbits][nrows_a][ncols_a/64] of uint64."""
        return self._info().data

    def isBipolar(self) -> bool:
        return bool(self._info().isbipolar)

    def wordsPerRow(self) -> int:
        return self.ncols_a // 64

    def wordsPerBitplane(self) -> int:
        return self.nrows_a * self.wordsPerRow()

    def importRegular(self, matrix, readColMajor: bool = False, stream=None) -> None:
        """importRegular<T> / importRegular(uint8_t*) (gemmbitserial.hpp:213, 249); T = int8, int16,
        int32 or float32."""
        ptr, dt, keep = _src(matrix, allow_float=True)
        _capi.check(_capi.load().gbs_import(self._ctx._h, self._side, ptr, dt, int(bool(readColMajor)),
                                            _stream_handle(stream)))
        _release(keep, matrix, stream)

    def importRegularAndQuantize(self, matrix, thresholds, nThres=None, readColMajor: bool = False,
                                 stream=None) -> None:
        """importRegularAndQuantize<T> (gemmbitserial.hpp:282-305): thresholds shaped [nThres][nrows],
        same element type as matrix (int8, uint8, int16, int32 or float32)."""
        ptr, dt, keep = _src(matrix, allow_float=True)
        if nThres is None:
            nThres = int(thresholds.shape[0]) if thresholds is not None and len(thresholds.shape) == 2 else 0
        if nThres:
            tptr, tdt, tkeep = _src(thresholds, allow_float=True)
            if tdt != dt:
                raise TypeError("thresholds must have the element type of the matrix")
        else:
            tptr, tkeep = None, None
        _capi.check(_capi.load().gbs_import_quantize(self._ctx._h, self._side, ptr, tptr, int(nThres), dt,
                                                     int(bool(readColMajor)), _stream_handle(stream)))
        _release(keep, matrix, stream)
        if tkeep is not None:
            _release(tkeep, thresholds, stream)

    # single bits (gemmbitserial.hpp:90-108); each call synchronises the device
    def get(self, bit: int, row: int, col: int) -> bool:
        v = C.c_int()
        _capi.check(_capi.load().gbs_get_bit(self._ctx._h, self._side, bit, row, col, C.byref(v)))
        return bool(v.value)

    def set(self, bit: int, row: int, col: int) -> None:
        _capi.check(_capi.load().gbs_set_bit(self._ctx._h, self._side, bit, row, col, 1))

    def unset(self, bit: int, row: int, col: int) -> None:
        _capi.check(_capi.load().gbs_set_bit(self._ctx._h, self._side, bit, row, col, 0))

    def clearAll(self, stream=None) -> None:
        _capi.check(_capi.load().gbs_clear(self._ctx._h, self._side, _stream_handle(stream)))

    def planes(self, stream=None) -> np.ndarray:
        """Host copy of the packed planes, shape [nbits, nrows_a, ncols_a/64] (uint64)."""
        i = self._info()
        shape = (int(i.nbits), int(i.nrows_a), int(i.ncols_a // 64))
        out = np.zeros(max(int(np.prod(shape)), 1), np.uint64)
        _capi.check(_capi.load().gbs_get_planes(self._ctx._h, self._side, C.c_void_p(out.ctypes.data),
                                                _stream_handle(stream)))
        return out[:int(np.prod(shape))].reshape(shape)

    def exportRegular(self, stream=None) -> np.ndarray:
        """exportRegular<int32_t> (gemmbitserial.hpp:313-333): rows x ncols int32 on the host."""
        out = np.zeros(max(self.nrows * self.ncols, 1), np.int32)
        _capi.check(_capi.load().gbs_export(self._ctx._h, self._side, C.c_void_p(out.ctypes.data),
                                            _stream_handle(stream)))
        return out[:self.nrows * self.ncols].reshape(self.nrows, self.ncols)


class GEMMContext:
    """GEMMContext (gemmbitserial.hpp:379-411).  Copies of the Python object share one context."""

    def __init__(self, handle):
        self._h = handle
        self.lhs = BitSerialMatrix(self, 0)
        self.rhs = BitSerialMatrix(self, 1)

    def _info(self):
        if not self._h:
            raise RuntimeError("context has been deallocated")
        info = _capi.CtxInfo()
        _capi.check(_capi.load().gbs_ctx_get_info(self._h, C.byref(info)))
        return info

    @property
    def lhsBlock(self): return self._info().lhsBlock

    @property
    def rhsBlock(self): return self._info().rhsBlock

    @property
    def res(self) -> np.ndarray:
        """ctx.res: the rhs.nrows x lhs.nrows int32 result, flattened (transposed layout)."""
        info = self._info()
        n = info.lhs.nrows * info.rhs.nrows
        out = np.zeros(max(n, 1), np.int32)
        _capi.check(_capi.load().gbs_get_result(self._h, C.c_void_p(out.ctypes.data), _stream_handle(None)))
        return out[:n]

    @property
    def res_device(self) -> int:
        return self._info().res

    def isBipolarTimesRegular(self) -> bool:
        return self.lhs.isBipolar() != self.rhs.isBipolar()

    def isBipolarTimesBipolar(self) -> bool:
        return self.lhs.isBipolar() and self.rhs.isBipolar()

    def isMatrixVector(self) -> bool:
        return self.rhs.nrows == 1

    def set_pipe(self, pipe: int) -> None:
        _capi.check(_capi.load().gbs_set_pipe(self._h, pipe))

    def set_host_import(self, mode: int) -> None:
        """GBS_HOST_IMPORT_AUTO (read host sources in place where the device can) or
        GBS_HOST_IMPORT_STAGED (copy-engine copies; for contexts whose imports run beside
        another context's GEMM)."""
        _capi.check(_capi.load().gbs_set_host_import(self._h, mode))

    @property
    def pipe(self) -> int:
        return self._info().pipe


def allocGEMMContext(lhsRows, depth, rhsRows, lhsBits, rhsBits, lhsSigned, rhsSigned) -> GEMMContext:
    """allocGEMMContext (arch-generic.hpp:78-100, gemmbitserial.hpp:415-452)."""
    h = C.c_void_p()
    _capi.check(_capi.load().gbs_ctx_alloc(int(lhsRows), int(depth), int(rhsRows), int(lhsBits), int(rhsBits),
                                           int(bool(lhsSigned)), int(bool(rhsSigned)), C.byref(h)))
    return GEMMContext(h)


allocateGEMMContext = allocGEMMContext  # the name README.md:15 uses


def gemmBitSerial(ctx: GEMMContext, stream=None, out=None) -> None:
    """gemmBitSerial (arch-generic.hpp:331-345); asynchronous on the stream.

    With `out` (a C-contiguous int32 numpy array or torch tensor of N*M
    elements, host or device), the result goes straight there (gbs_gemm_to)
    and the call returns once it has landed when `out` is in host memory;
    ctx.res is then stale until the next plain call."""
    lib = _capi.load()
    if out is None:
        _capi.check(lib.gbs_gemm(ctx._h, _stream_handle(stream)))
        return
    info = ctx._info()
    n = info.lhs.nrows * info.rhs.nrows
    if hasattr(out, "data_ptr"):
        import torch
        if out.dtype != torch.int32 or not out.is_contiguous() or out.numel() < n:
            raise ValueError("out must be a contiguous int32 tensor of at least N*M elements")
        ptr = out.data_ptr()
    else:
        if out.dtype != np.int32 or not out.flags["C_CONTIGUOUS"] or out.size < n:
            raise ValueError("out must be a C-contiguous int32 array of at least N*M elements")
        ptr = out.ctypes.data
    _capi.check(lib.gbs_gemm_to(ctx._h, C.c_void_p(ptr), _stream_handle(stream)))


def deallocGEMMContext(ctx: GEMMContext) -> None:
    """deallocGEMMContext (gemmbitserial.hpp:454-458)."""
    if ctx._h:
        _capi.check(_capi.load().gbs_ctx_free(ctx._h))
        ctx._h = None


def sumRows(m: BitSerialMatrix, stream=None) -> np.ndarray:
    """sumRows (arch-generic.hpp:6-37): per-row sum of the values of one operand."""
    out = np.zeros(max(m.nrows, 1), np.int32)
    _capi.check(_capi.load().gbs_sum_rows(m._ctx._h, m._side, C.c_void_p(out.ctypes.data), _stream_handle(stream)))
    return out[:m.nrows]
