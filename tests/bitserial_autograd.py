"""Thin ctypes test binding: the bit-serial GEMM as a torch.autograd.Function.

Forward: exact int32 bit-serial GEMM through the C ABI (returned as float32,
exact while |res| < 2^24).  Backward: gbs_adjoint, the FP32 gradients with
respect to the VALUES the packed operands encode (straight-through w.r.t. the
int8 inputs, as quantisation-aware training uses them).
"""
import ctypes as C

import torch

from gemmbitserial_gb300 import _capi
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial


class BitSerialMatmul(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, B, wA, sA, wB, sB):
        """A: M x K, B: N x K CUDA tensors holding the quantised integer values
        (float or integer dtype); returns res = B.A^T as N x M float32."""
        M, K = A.shape
        N = B.shape[0]
        g = allocGEMMContext(M, K, N, wA, wB, sA, sB)
        s = torch.cuda.current_stream()
        g.lhs.importRegular(A.detach().round().to(torch.int8).contiguous(), stream=s)
        g.rhs.importRegular(B.detach().round().to(torch.int8).contiguous(), stream=s)
        gemmBitSerial(g, stream=s)
        res = torch.empty(N, M, dtype=torch.int32, device=A.device)
        _capi.check(_capi.load().gbs_get_result(g._h, C.c_void_p(res.data_ptr()), C.c_void_p(s.cuda_stream)))
        ctx.g = g
        ctx.shape = (M, K, N)
        return res.float()

    @staticmethod
    def backward(ctx, dC):
        M, K, N = ctx.shape
        g = ctx.g
        dC = dC.contiguous().float()
        dA = torch.empty(M, K, dtype=torch.float32, device=dC.device) if ctx.needs_input_grad[0] else None
        dB = torch.empty(N, K, dtype=torch.float32, device=dC.device) if ctx.needs_input_grad[1] else None
        s = torch.cuda.current_stream()
        _capi.check(_capi.load().gbs_adjoint(
            g._h, C.c_void_p(dC.data_ptr()), C.c_void_p(dA.data_ptr() if dA is not None else 0),
            C.c_void_p(dB.data_ptr() if dB is not None else 0), C.c_void_p(s.cuda_stream)))
        s.synchronize()
        deallocGEMMContext(g)
        return dA, dB, None, None, None, None
