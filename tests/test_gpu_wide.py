"""5- to 8-bit operands on the tensor cores: each wide operand splits by planes
into a low (unsigned) and a high part of at most 4 bits, every part product
runs as an exact digit GEMM, and the shifted partial results add up in 32-bit
wrap-around arithmetic.  Bit-exact against the oracle for every width and
encoding pair, on the persistent one-problem kernel (a side under 256) and the
SM-pair kernels, after re-imports, and at full size."""
import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from oracle import oracle as O

pytestmark = pytest.mark.gpu

WIDE = [(5, "u"), (5, "s"), (6, "s"), (7, "u"), (8, "u"), (8, "s")]
NARROW = [(1, "b"), (2, "s"), (4, "u")]


def run(A, B, wa, ea, wb, eb, pipe=_capi.GBS_PIPE_AUTO):
    M, K = A.shape
    N = B.shape[0]
    ctx = allocGEMMContext(M, K, N, wa, wb, ea != "u", eb != "u")
    try:
        ctx.set_pipe(pipe)
        if pipe == _capi.GBS_PIPE_TC:
            assert ctx.pipe == _capi.GBS_PIPE_TC, "the wide path applies"
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        return ctx.res.reshape(N, M).copy()
    finally:
        deallocGEMMContext(ctx)


@pytest.mark.parametrize("shape", [(96, 1000, 80), (300, 640, 520), (257, 2048, 300)],
                         ids=["96x1000x80", "300x640x520", "257x2048x300"])
def test_wide_encodings_vs_oracle(shape):
    M, K, N = shape
    rng = np.random.default_rng(M + K + N)
    pairs = [(a, b) for a in WIDE for b in WIDE + NARROW] + [(a, b) for a in NARROW for b in WIDE]
    for (wa, ea), (wb, eb) in pairs:
        A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
        got = run(A, B, wa, ea, wb, eb, pipe=_capi.GBS_PIPE_TC)
        assert np.array_equal(got, O.oracle_gemm(A, B, wa, wb, ea != "u", eb != "u")), (shape, wa, ea, wb, eb)
    assert _capi.load().gbs_debug_tc_error() == 0


def test_wide_follows_reimports():
    """The parts' digit matrices are rebuilt after an import changes the planes."""
    M, K, N = 512, 1024, 384
    rng = np.random.default_rng(3)
    A1 = datagen.operand(int(rng.integers(1 << 30)), M, K, 8, "s")
    A2 = datagen.operand(int(rng.integers(1 << 30)), M, K, 8, "s")
    B = datagen.operand(int(rng.integers(1 << 30)), N, K, 6, "u")
    ctx = allocGEMMContext(M, K, N, 8, 6, True, False)
    try:
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        ctx.lhs.importRegular(A1)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), O.oracle_gemm(A1, B, 8, 6, True, False))
        ctx.lhs.importRegular(A2)
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), O.oracle_gemm(A2, B, 8, 6, True, False))
    finally:
        deallocGEMMContext(ctx)


@pytest.mark.parametrize("enc", ["u", "s"])
def test_wide_full_size_8bit(enc):
    """2048 x 4096 x 2048 at 8 x 8 bits: the automatic choice runs the tensor cores, bit-exact."""
    M, K, N = 2048, 4096, 2048
    A = datagen.operand(datagen.SEED_BASE + 970, M, K, 8, enc)
    B = datagen.operand(datagen.SEED_BASE + 971, N, K, 8, enc)
    ctx = allocGEMMContext(M, K, N, 8, 8, enc == "s", enc == "s")
    try:
        assert ctx.pipe == _capi.GBS_PIPE_TC
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        got = ctx.res.reshape(N, M)
    finally:
        deallocGEMMContext(ctx)
    assert np.array_equal(got, O.oracle_gemm(A, B, 8, 8, enc == "s", enc == "s", threads=16))


def test_wide_beyond_the_bound_stays_on_the_cuda_cores():
    """K * 15 * 15 >= 2^24: a part product could leave the exact fp32 range, so the tensor pipe declines."""
    ctx = allocGEMMContext(128, 80000, 128, 8, 8, False, False)
    try:
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        assert ctx.pipe == _capi.GBS_PIPE_POPC
    finally:
        deallocGEMMContext(ctx)
