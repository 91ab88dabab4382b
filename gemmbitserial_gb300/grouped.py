"""Grouped bit-serial GEMM: many contexts in one persistent launch (C ABI gbs_group_*).

The reference runs a list of GEMMs as a host loop of gemmBitSerial over a
vector of contexts (benchmark.cpp:192-219); a Group runs the same list as one
persistent kernel draining a device tile queue, optionally captured together
with the packing of every operand into one CUDA graph.
"""
from __future__ import annotations

import ctypes as C

from . import _capi
from .api import _stream_handle


def _dtype_code(t):
    import torch
    return {torch.int8: _capi.GBS_I8, torch.uint8: _capi.GBS_U8,
            torch.int16: _capi.GBS_I16, torch.int32: _capi.GBS_I32}[t.dtype]


class Group:
    def __init__(self, ctxs):
        self.ctxs = list(ctxs)
        arr = (C.c_void_p * max(1, len(self.ctxs)))(*[c._h for c in self.ctxs])
        self._h = C.c_void_p()
        _capi.check(_capi.load().gbs_group_create(arr, len(self.ctxs), C.byref(self._h)))
        self._keep = None

    def _srcs(self, lhs, rhs):
        n = len(self.ctxs)
        L = (C.c_void_p * n)(*[t.data_ptr() for t in lhs])
        R = (C.c_void_p * n)(*[t.data_ptr() for t in rhs])
        D = (C.c_int * (2 * n))(*[v for a, b in zip(lhs, rhs) for v in (_dtype_code(a), _dtype_code(b))])
        return L, R, D

    def import_(self, lhs, rhs, stream=None):
        """Packs every operand (row-major CUDA tensors: lhs[p] M x K, rhs[p] N x K) in one launch."""
        L, R, D = self._srcs(lhs, rhs)
        _capi.check(_capi.load().gbs_group_import(self._h, L, R, D, _stream_handle(stream)))

    def gemm(self, stream=None):
        _capi.check(_capi.load().gbs_group_gemm(self._h, _stream_handle(stream)))

    def capture(self, lhs=None, rhs=None, stream=None):
        """Captures [grouped import] + grouped GEMM into a CUDA graph (stream must not be the legacy default)."""
        if lhs is None:
            _capi.check(_capi.load().gbs_group_capture(self._h, None, None, None, _stream_handle(stream)))
        else:
            L, R, D = self._srcs(lhs, rhs)
            self._keep = (lhs, rhs)
            _capi.check(_capi.load().gbs_group_capture(self._h, L, R, D, _stream_handle(stream)))

    def replay(self, stream=None):
        _capi.check(_capi.load().gbs_group_replay(self._h, _stream_handle(stream)))

    def status(self, stream=None):
        return _capi.load().gbs_group_status(self._h, _stream_handle(stream))

    def stats(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _capi.check(_capi.load().gbs_group_stats(self._h, C.byref(a), C.byref(b), C.byref(c)))
        d, e, f = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _capi.check(_capi.load().gbs_group_split(self._h, C.byref(d), C.byref(e), C.byref(f)))
        return {"tiles": a.value, "smem_bytes": b.value, "grid": c.value,
                "popc_problems": d.value, "tc_problems": e.value, "tc_tiles": f.value,
                "tc_kernel": ("none", "digits", "nibbles")[_capi.load().gbs_debug_group_tc_kernel(self._h)]}

    def free(self):
        if self._h:
            _capi.check(_capi.load().gbs_group_free(self._h))
            self._h = None
