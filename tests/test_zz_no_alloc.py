"""gbs_gemm_noalloc: the one-shot GEMM for callers that cannot let the library
allocate (graph capture in global mode, real-time loops, fixed memory
budgets).  It works in a fixed file-scope device array instead of cudaMalloc.
Its results must equal the context path's (alloc -> import -> gemm) bit for
bit, on consecutive calls that reuse the shared array with different shapes
and encodings.  This file sorts last so a stop-at-first-failure run has run
every other test before it."""
import ctypes as C

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial

pytestmark = pytest.mark.gpu

# consecutive calls: bipolar x regular (uses the row-sum part of the array),
# then a larger multi-bit GEMM, then a small one over the stale contents
CALLS = [(300, 1000, 200, 1, "b", 4, "s"), (2048, 4096, 2048, 3, "u", 2, "s"), (17, 70, 5, 2, "s", 1, "b")]


def context_path(A, B, wA, eA, wB, eB):
    M, K = A.shape
    N = B.shape[0]
    ctx = allocGEMMContext(M, K, N, wA, wB, eA != "u", eB != "u")
    try:
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        return ctx.res.reshape(N, M)
    finally:
        deallocGEMMContext(ctx)


def test_noalloc_matches_context_path_on_consecutive_calls(gbs_lib):
    import torch
    assert torch.cuda.is_available()
    stream = torch.cuda.Stream()
    for i, (M, K, N, wA, eA, wB, eB) in enumerate(CALLS):
        A = datagen.operand(datagen.SEED_BASE + 300 + 2 * i, M, K, wA, eA)
        B = datagen.operand(datagen.SEED_BASE + 301 + 2 * i, N, K, wB, eB)
        dA = torch.from_numpy(A).cuda()
        dB = torch.from_numpy(B).cuda()
        res = torch.full((N, M), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = gbs_lib.gbs_gemm_noalloc(C.c_void_p(dA.data_ptr()), _capi.GBS_I8, C.c_void_p(dB.data_ptr()), _capi.GBS_I8,
                                      M, K, N, wA, wB, int(eA != "u"), int(eB != "u"), C.c_void_p(res.data_ptr()),
                                      C.c_void_p(stream.cuda_stream))
        assert rc == _capi.GBS_OK, gbs_lib.gbs_last_error()
        stream.synchronize()
        assert np.array_equal(res.cpu().numpy(), context_path(A, B, wA, eA, wB, eB)), CALLS[i]


def test_noalloc_rejects_what_does_not_fit(gbs_lib):
    import torch
    cap = gbs_lib.gbs_noalloc_scratch_bytes()
    assert cap == 16 << 20
    x = torch.zeros(16, dtype=torch.int8, device="cuda")
    r = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = gbs_lib.gbs_gemm_noalloc(C.c_void_p(x.data_ptr()), 0, C.c_void_p(x.data_ptr()), 0, 8192, 8192, 8192,
                                  8, 8, 0, 0, C.c_void_p(r.data_ptr()), None)
    assert rc == _capi.GBS_EINVAL
    assert b"fixed array holds" in gbs_lib.gbs_last_error()
    host = np.zeros(64, np.int8)
    rc = gbs_lib.gbs_gemm_noalloc(C.c_void_p(host.ctypes.data), 0, C.c_void_p(host.ctypes.data), 0, 4, 16, 4,
                                  1, 1, 0, 0, C.c_void_p(r.data_ptr()), None)
    assert rc == _capi.GBS_EINVAL
