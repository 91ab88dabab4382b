"""gbs_gemm_noalloc: the one-shot GEMM for callers that cannot let the library
allocate (graph capture in global mode, real-time loops, fixed memory
budgets).  It works in a fixed file-scope device array instead of cudaMalloc.
Its results must equal the oracle's and the context path's (alloc -> import ->
gemm) bit for bit, on consecutive calls that reuse the shared array with
different shapes and encodings.  This file sorts last so a stop-at-first-failure
run has run every other test before it."""
import ctypes as C

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# consecutive calls: bipolar x regular (uses the row-sum part of the array),
# then a larger multi-bit GEMM, then a small one over the stale contents, then
# bipolar x bipolar with K % 256 != 0 after the larger call: its result
# (ncols - 2*popc(a ^ b)) is only right if the column padding of the reused
# array reads as zero in both operands
CALLS = [(300, 1000, 200, 1, "b", 4, "s"), (2048, 4096, 2048, 3, "u", 2, "s"), (17, 70, 5, 2, "s", 1, "b"),
         (2048, 4096, 2048, 4, "u", 4, "u"), (129, 333, 77, 1, "b", 1, "b"), (64, 8000, 3, 1, "b", 1, "b")]


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


def test_noalloc_matches_oracle_on_consecutive_calls(gbs_lib):
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
        got = res.cpu().numpy()
        want = O.oracle_gemm(A, B, wA, wB, eA != "u", eB != "u", threads=8)
        assert np.array_equal(got, want), CALLS[i]
        assert np.array_equal(got, context_path(A, B, wA, eA, wB, eB)), CALLS[i]


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


def test_noalloc_rejects_memory_of_other_devices(gbs_lib):
    """The pointer checks run on the host before any launch: host memory, and
    (where a second GPU is visible) another GPU's memory, return GBS_EINVAL and
    leave the result untouched."""
    import torch
    r = torch.full((16,), 7, dtype=torch.int32, device="cuda:0")
    host = np.zeros(64, np.int8)
    torch.cuda.synchronize()
    rc = gbs_lib.gbs_gemm_noalloc(C.c_void_p(host.ctypes.data), 0, C.c_void_p(host.ctypes.data), 0, 4, 16, 4,
                                  1, 1, 0, 0, C.c_void_p(r.data_ptr()), None)
    assert rc == _capi.GBS_EINVAL
    assert b"current device" in gbs_lib.gbs_last_error()
    if torch.cuda.device_count() >= 2:
        other = torch.zeros(64, dtype=torch.int8, device="cuda:1")
        mine = torch.zeros(64, dtype=torch.int8, device="cuda:0")
        for lhs, rhs in ((other, mine), (mine, other)):
            rc = gbs_lib.gbs_gemm_noalloc(C.c_void_p(lhs.data_ptr()), 0, C.c_void_p(rhs.data_ptr()), 0, 4, 16, 4,
                                          1, 1, 0, 0, C.c_void_p(r.data_ptr()), None)
            assert rc == _capi.GBS_EINVAL
    torch.cuda.synchronize()
    assert (r.cpu() == 7).all()
