"""The rest of the drop-in surface on the GPU: float input through importRegular
(quantize<float>, gemmbitserial.hpp:170-186) against the reference's own results,
and the single-bit accessors get / set / unset / clearAll (:90-108), including that
a GEMM after bit edits sees them on every pipe."""
import ctypes as C
import os

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PIPES = [_capi.GBS_PIPE_AUTO, _capi.GBS_PIPE_POPC, _capi.GBS_PIPE_BMMA, _capi.GBS_PIPE_TC]


@pytest.fixture(scope="module", autouse=True)
def lib(gbs_lib):
    import torch
    assert torch.cuda.is_available()
    return gbs_lib


def export(ctx, side, rows, cols):
    out = np.zeros((rows, cols), np.int32)
    if rows * cols:
        _capi.check(_capi.load().gbs_export(ctx._h, side, C.c_void_p(out.ctypes.data), None))
    return out


@pytest.mark.parametrize("device", [False, True], ids=["host", "device"])
def test_float_import_matches_reference(device):
    import torch
    z = np.load(os.path.join(GOLD, "ref_float_import.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    for k in keys:
        src, want = z[k + "_src"], z[k + "_values"]
        bits, sgn = (int(x) for x in z[k + "_meta"])
        rows, cols = src.shape
        ctx = allocGEMMContext(rows, cols, 1, bits, 1, bool(sgn), False)
        try:
            ctx.lhs.importRegular(torch.from_numpy(src).cuda() if device else src)
            torch.cuda.synchronize()
            assert np.array_equal(export(ctx, 0, rows, cols), want), k
        finally:
            deallocGEMMContext(ctx)


@pytest.mark.parametrize("pipe", PIPES)
def test_float_operands_gemm(pipe):
    rng = np.random.default_rng(11)
    for (M, K, N, wa, sa, wb, sb, cm) in [(300, 700, 260, 3, True, 2, False, False), (64, 128, 70, 1, True, 4, True, True),
                                          (17, 333, 5, 2, False, 1, True, False)]:
        def draw(rows, w, s):
            if w == 1 and s:
                return rng.uniform(-2, 2, (rows, K)).astype(np.float32)
            lo, hi = (-(1 << (w - 1)), 1 << (w - 1)) if s else (0, 1 << w)
            return rng.uniform(lo, hi - 1e-3, (rows, K)).astype(np.float32)
        A, B = draw(M, wa, sa), draw(N, wb, sb)
        want = O.oracle_gemm(O.import_values(A, wa, sa).astype(np.int8), O.import_values(B, wb, sb).astype(np.int8),
                             wa, wb, sa, sb)
        ctx = allocGEMMContext(M, K, N, wa, wb, sa, sb)
        try:
            ctx.set_pipe(pipe)
            ctx.lhs.importRegular(np.ascontiguousarray(A.T) if cm else A, readColMajor=cm)
            ctx.rhs.importRegular(B)
            gemmBitSerial(ctx)
            assert np.array_equal(ctx.res.reshape(N, M), want), (M, K, N, pipe)
        finally:
            deallocGEMMContext(ctx)


def test_bits_get_set_unset_clear(lib):
    M, K, N = 70, 300, 40
    ctx = allocGEMMContext(M, K, N, 3, 1, False, False)
    try:
        A = datagen.operand(datagen.SEED_BASE + 1200, M, K, 3, "u")
        ctx.lhs.importRegular(A)
        for (b, r, c) in [(0, 0, 0), (2, 69, 299), (1, 33, 64), (0, 5, 63)]:
            assert ctx.lhs.get(b, r, c) == bool((int(A[r, c]) >> b) & 1)
        ctx.lhs.clearAll()
        assert not np.any(export(ctx, 0, M, K))
        want = np.zeros((M, K), np.int32)
        for (b, r, c) in [(0, 0, 0), (2, 69, 299), (1, 33, 64), (0, 5, 63), (2, 5, 63)]:
            ctx.lhs.set(b, r, c)
            want[r, c] |= 1 << b
        ctx.lhs.unset(2, 5, 63)
        want[5, 63] &= ~4
        assert np.array_equal(export(ctx, 0, M, K), want)
        assert ctx.lhs.get(2, 69, 299) and not ctx.lhs.get(2, 5, 63)
        # out of range, and the padding, are rejected
        assert lib.gbs_set_bit(ctx._h, 0, 3, 0, 0, 1) == _capi.GBS_EINVAL
        assert lib.gbs_set_bit(ctx._h, 0, 0, M, 0, 1) == _capi.GBS_EINVAL
        assert lib.gbs_set_bit(ctx._h, 0, 0, 0, K, 1) == _capi.GBS_EINVAL
        v = C.c_int(7)
        assert lib.gbs_get_bit(ctx._h, 0, 0, 0, K, C.byref(v)) == _capi.GBS_OK and v.value == 0  # padding reads 0
    finally:
        deallocGEMMContext(ctx)


@pytest.mark.parametrize("pipe", PIPES)
def test_gemm_sees_bit_edits(pipe):
    """Bit edits after a GEMM invalidate every derived operand (the tensor-core digits)."""
    M, K, N = 256, 512, 300
    A = datagen.operand(datagen.SEED_BASE + 1300, M, K, 2, "u")
    B = datagen.operand(datagen.SEED_BASE + 1301, N, K, 2, "s")
    ctx = allocGEMMContext(M, K, N, 2, 2, False, True)
    try:
        ctx.set_pipe(pipe)
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), O.oracle_gemm(A, B, 2, 2, False, True))
        A2 = A.copy()
        for (r, c) in [(0, 0), (100, 511), (255, 17)]:
            for b in range(2):
                if (A2[r, c] >> b) & 1:
                    ctx.lhs.unset(b, r, c)
                else:
                    ctx.lhs.set(b, r, c)
            A2[r, c] ^= 3
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), O.oracle_gemm(A2, B, 2, 2, False, True))
        ctx.rhs.clearAll()
        gemmBitSerial(ctx)
        assert not np.any(ctx.res)
    finally:
        deallocGEMMContext(ctx)


def test_word_get_set_through_the_abi(gbs_lib):
    """gbs_get_word / gbs_set_word (BitSerialMatrix::word): one device word; padding stays zero, and a
    GEMM after a word write sees the new bits."""
    import ctypes as C
    lib = gbs_lib
    M, K, N = 40, 100, 30
    A = datagen.operand(datagen.SEED_BASE + 990, M, K, 2, "u")
    B = datagen.operand(datagen.SEED_BASE + 991, N, K, 1, "u")
    ctx = allocGEMMContext(M, K, N, 2, 1, False, False)
    try:
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        v = C.c_uint64()
        _capi.check(lib.gbs_get_word(ctx._h, 0, 1, 7, 70, C.byref(v)))
        want = sum(((int(A[7, c]) >> 1) & 1) << (c - 64) for c in range(64, K))
        assert v.value == want
        _capi.check(lib.gbs_set_word(ctx._h, 0, 1, 7, 70, 0xFFFFFFFFFFFFFFFF))
        _capi.check(lib.gbs_get_word(ctx._h, 0, 1, 7, 70, C.byref(v)))
        assert v.value == (1 << (K - 64)) - 1  # columns past K stay zero
        A2 = A.copy()
        A2[7, 64:] |= 2
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), O.oracle_gemm(A2, B, 2, 1, False, False))
    finally:
        deallocGEMMContext(ctx)
