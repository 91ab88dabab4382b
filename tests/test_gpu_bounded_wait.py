"""Failure handling of the tensor-core kernels, tested without a GPU fault: a
bounded mbarrier wait that nothing will complete (no copy and no MMA was
issued) gives up after a short limit, the kernel drains, frees TMEM and
returns, and the host reads GBS_ETIMEOUT; the context and the GPU stay usable."""
import ctypes as C

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_the_context_stays_usable(gbs_lib):
    lib = gbs_lib
    M, K, N = 512, 1024, 512
    A = datagen.operand(datagen.SEED_BASE + 950, M, K, 3, "u")
    B = datagen.operand(datagen.SEED_BASE + 951, N, K, 2, "s")
    ctx = allocGEMMContext(M, K, N, 3, 2, False, True)
    try:
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        for _ in range(2):  # the hook leaves nothing behind: a second run behaves the same
            rc = lib.gbs_debug_tc_timeout(ctx._h, 64, None)
            assert rc == _capi.GBS_ETIMEOUT, lib.gbs_last_error()
            assert b"gave up" in lib.gbs_last_error()
            assert lib.gbs_debug_tc_error() == 0  # cleared again
        # the same context, on the same kernel, right after: bit-exact
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        _capi.check(lib.gbs_set_variant(ctx._h, 2561))
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), O.oracle_gemm(A, B, 3, 2, False, True))
        assert lib.gbs_debug_tc_error() == 0
    finally:
        deallocGEMMContext(ctx)


def test_bounded_wait_hook_rejects_what_it_cannot_run(gbs_lib):
    lib = gbs_lib
    ctx = allocGEMMContext(64, 256, 64, 2, 2, False, False)
    try:
        assert lib.gbs_debug_tc_timeout(ctx._h, 64, None) == _capi.GBS_ESTATE  # not imported
        ctx.lhs.importRegular(np.zeros((64, 256), np.int8))
        ctx.rhs.importRegular(np.zeros((64, 256), np.int8))
        assert lib.gbs_debug_tc_timeout(ctx._h, 64, None) == _capi.GBS_EUNSUPPORTED  # too small for SM pairs
        assert lib.gbs_debug_tc_timeout(ctx._h, 0, None) == _capi.GBS_EINVAL
    finally:
        deallocGEMMContext(ctx)
