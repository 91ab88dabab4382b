"""The 5th-generation tensor-core pipe (tcgen05.mma on plane pairs as fp8
{0, +-2^i} operands, TMEM accumulation): bit-exact against the oracle and
the reference's own full-size results, including sums up to just below 2^24
(the exactness bound the pipe is selected under)."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CFG = json.load(open(os.path.join(GOLD, "ref_configs.json")))


@pytest.fixture(scope="module", autouse=True)
def lib(gbs_lib):
    import torch
    assert torch.cuda.is_available()
    return gbs_lib


PAIR = (_capi.GBS_PIPE_TC, 512)  # 256 x 256 tiles on SM pairs
PAIR128 = (_capi.GBS_PIPE_TC, 513)  # 256 x 128 tiles on SM pairs


def tc_gemm(A, B, wA, wB, sA, sB, expect_tc=True, pipe=_capi.GBS_PIPE_TC):
    M, K = A.shape
    N = B.shape[0]
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    try:
        if isinstance(pipe, tuple):
            pipe, variant = pipe
            _capi.check(_capi.load().gbs_set_variant(ctx._h, variant))
        ctx.set_pipe(pipe)
        if expect_tc:
            wpr = -(-K // 64) if N != 1 else -(-K // 256) * 4  # the reference's words per plane row
            if pipe in (_capi.GBS_PIPE_TC_SMEM, _capi.GBS_PIPE_TC_PAIRS) and (wpr % 2 or max(wA, wB) > 4):
                # odd word counts and operands wider than one digit: the shared-memory variants decline
                assert ctx.pipe == _capi.GBS_PIPE_POPC
            else:
                assert ctx.pipe == pipe, "tensor-core pipe not applicable"
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        return ctx.res.reshape(N, M)
    finally:
        deallocGEMMContext(ctx)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_tc_small_first():
    A = datagen.operand(datagen.SEED_BASE + 500, 128, 256, 1, "u")
    B = datagen.operand(datagen.SEED_BASE + 501, 128, 256, 1, "u")
    got = tc_gemm(A, B, 1, 1, False, False)
    assert _capi.load().gbs_debug_tc_error() == 0
    assert np.array_equal(got, O.oracle_gemm(A, B, 1, 1, False, False))


ENCS = [(1, "u"), (1, "b"), (2, "u"), (2, "s"), (3, "u"), (3, "s"), (4, "u"), (4, "s")]


MODES = [_capi.GBS_PIPE_TC, PAIR, PAIR128, _capi.GBS_PIPE_TC_SMEM, _capi.GBS_PIPE_TC_PAIRS]
MODE_IDS = ["hbm-digits", "hbm-digits-sm-pair", "hbm-digits-sm-pair-128", "smem-digits", "plane-pairs"]


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
@pytest.mark.parametrize("shape", [(128, 256, 128), (200, 1000, 333), (64, 128, 64), (300, 3000, 129),
                                   (129, 64, 700), (256, 512, 520)])
def test_tc_encodings_vs_oracle(shape, mode):
    M, K, N = shape
    rng = np.random.default_rng(M + K + N)
    for (wa, ea) in ENCS:
        for (wb, eb) in ENCS:
            if wa + wb > 5:
                continue
            A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
            B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
            sa, sb = ea != "u", eb != "u"
            assert np.array_equal(tc_gemm(A, B, wa, wb, sa, sb, pipe=mode), O.oracle_gemm(A, B, wa, wb, sa, sb)), \
                (shape, wa, ea, wb, eb)
    assert _capi.load().gbs_debug_tc_error() == 0


@pytest.mark.parametrize("mode", MODES, ids=MODE_IDS)
@pytest.mark.parametrize("name", sorted(CFG))
def test_tc_full_size_workloads(name, mode):
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
    assert sha(tc_gemm(A, B, wA, wB, sA, sB, expect_tc=min(M, N) >= 64, pipe=mode)) == CFG[name]["sha256"]


def test_tc_sums_near_the_exactness_bound():
    """4-bit x 1-bit unsigned, every product 15: sums of 15 * K with K = 1,118,464 - 64 stay < 2^24."""
    M, N = 128, 128
    K = (1 << 24) // 15 - 64
    A = np.full((M, K), 15, np.int8)
    B = np.ones((N, K), np.int8)
    B[1::2, ::3] = 0
    want = O.oracle_gemm(A, B, 4, 1, False, False, threads=16)
    A2 = np.where((np.arange(K) // 7) % 2 == 0, -8, 7).astype(np.int8)[None, :].repeat(M, 0)
    want2 = O.oracle_gemm(A2, B, 4, 1, True, False, threads=16)
    for mode in MODES:
        assert np.array_equal(tc_gemm(A, B, 4, 1, False, False, pipe=mode), want)
        # signed: alternating -8 / +7 partial sums swing across zero
        assert np.array_equal(tc_gemm(A2, B, 4, 1, True, False, pipe=mode), want2)
    assert _capi.load().gbs_debug_tc_error() == 0


def test_tc_pipe_declines_what_it_cannot_do_exactly():
    """K beyond the fp32 bound falls back to the CUDA-core pipe (8-bit operands run in plane parts
    on the digit pipe, but not on the shared-memory variants); the shared-memory variants also
    decline more than 5 planes; AUTO keeps tiny problems on the CUDA cores."""
    ctx = allocGEMMContext(128, 1 << 21, 128, 4, 1, False, False)
    ctx.set_pipe(_capi.GBS_PIPE_TC)
    assert ctx.pipe == _capi.GBS_PIPE_POPC
    deallocGEMMContext(ctx)
    ctx = allocGEMMContext(128, 256, 128, 8, 1, False, False)
    ctx.set_pipe(_capi.GBS_PIPE_TC)
    assert ctx.pipe == _capi.GBS_PIPE_TC
    ctx.set_pipe(_capi.GBS_PIPE_TC_SMEM)
    assert ctx.pipe == _capi.GBS_PIPE_POPC
    deallocGEMMContext(ctx)
    ctx = allocGEMMContext(128, 256, 128, 4, 4, False, False)
    ctx.set_pipe(_capi.GBS_PIPE_TC_SMEM)
    assert ctx.pipe == _capi.GBS_PIPE_POPC
    ctx.set_pipe(_capi.GBS_PIPE_TC)
    assert ctx.pipe == _capi.GBS_PIPE_TC
    deallocGEMMContext(ctx)
    ctx = allocGEMMContext(128, 320, 128, 2, 2, False, False)  # 5 plane words per row: 128-bit stages do not fit
    ctx.set_pipe(_capi.GBS_PIPE_TC_SMEM)
    assert ctx.pipe == _capi.GBS_PIPE_POPC
    ctx.set_pipe(_capi.GBS_PIPE_TC)
    assert ctx.pipe == _capi.GBS_PIPE_TC
    deallocGEMMContext(ctx)
    ctx = allocGEMMContext(4, 256, 2, 1, 1, False, False)
    assert ctx.pipe == _capi.GBS_PIPE_POPC
    deallocGEMMContext(ctx)


@pytest.mark.parametrize("shape", [(1, 4096, 3000, 4, "u", 4, "s"), (17, 333, 129, 2, "u", 1, "b"),
                                   (200, 1000, 96, 3, "s", 2, "u"), (255, 640, 255, 4, "u", 4, "u"),
                                   (64, 100, 4096, 1, "b", 1, "b")])
def test_tc_persistent_single_problem(shape):
    """Shapes with a side under 256 rows run the persistent kernel over a one-problem plan."""
    M, K, N, wa, ea, wb, eb = shape
    A = datagen.operand(datagen.SEED_BASE + 700 + M, M, K, wa, ea)
    B = datagen.operand(datagen.SEED_BASE + 701 + N, N, K, wb, eb)
    got = tc_gemm(A, B, wa, wb, ea != "u", eb != "u")
    assert np.array_equal(got, O.oracle_gemm(A, B, wa, wb, ea != "u", eb != "u"))
    assert _capi.load().gbs_debug_tc_error() == 0


def test_tc_peaks_probe():
    import ctypes as C
    f8, bf = C.c_double(), C.c_double()
    _capi.check(_capi.load().gbs_tc_peaks(C.byref(f8), C.byref(bf)))
    print(f"tcgen05 e4m3 {f8.value / 1e12:.0f} TFLOP/s, bf16 {bf.value / 1e12:.0f} TFLOP/s")
    assert f8.value > 1e14 and bf.value > 1e14
    assert _capi.load().gbs_debug_tc_error() == 0


def test_tc_digit_cache_follows_reimport():
    """The digit matrices are rebuilt after an import changes the planes."""
    M, K, N = 256, 640, 384
    A1 = datagen.operand(datagen.SEED_BASE + 610, M, K, 2, "u")
    A2 = datagen.operand(datagen.SEED_BASE + 611, M, K, 2, "u")
    B = datagen.operand(datagen.SEED_BASE + 612, N, K, 3, "s")
    ctx = allocGEMMContext(M, K, N, 2, 3, False, True)
    try:
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        ctx.lhs.importRegular(A1)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), O.oracle_gemm(A1, B, 2, 3, False, True))
        ctx.lhs.importRegular(A2)
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), O.oracle_gemm(A2, B, 2, 3, False, True))
    finally:
        deallocGEMMContext(ctx)


def last_pair(ctx, with_persistent=False):
    bn, sp, pe = C.c_int(0), C.c_int(0), C.c_int(0)
    _capi.check(_capi.load().gbs_debug_last_pair(ctx._h, C.byref(bn), C.byref(sp), C.byref(pe)))
    return (bn.value, sp.value, pe.value) if with_persistent else (bn.value, sp.value)


# (variant, M, K, N, expected K split): 1, 2 and 4 pairs per tile at both tile widths
SPLIT_CASES = [(512, 256, 8192, 256, 4), (512, 512, 2048, 512, 2), (512, 512, 512, 512, 1),
               (513, 256, 8192, 256, 4), (513, 512, 2048, 512, 2), (513, 256, 512, 256, 1)]


@pytest.mark.parametrize("case", SPLIT_CASES, ids=[f"v{c[0]}-{c[1]}x{c[2]}x{c[3]}" for c in SPLIT_CASES])
def test_pair_split_k(case):
    """The SM-pair kernel's in-cluster K split (partials summed over distributed shared memory)."""
    variant, M, K, N, want_splits = case
    rng = np.random.default_rng(M * 7 + K + N + variant)
    for (wa, ea, wb, eb) in [(3, "u", 2, "s"), (1, "b", 1, "b"), (4, "s", 1, "b"), (2, "u", 1, "u")]:
        A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
        sa, sb = ea != "u", eb != "u"
        ctx = allocGEMMContext(M, K, N, wa, wb, sa, sb)
        try:
            _capi.check(_capi.load().gbs_set_variant(ctx._h, variant))
            ctx.set_pipe(_capi.GBS_PIPE_TC)
            assert ctx.pipe == _capi.GBS_PIPE_TC
            ctx.lhs.importRegular(A)
            ctx.rhs.importRegular(B)
            gemmBitSerial(ctx)
            got = ctx.res.reshape(N, M)
            assert last_pair(ctx) == (256 if variant == 512 else 128, want_splits)
        finally:
            deallocGEMMContext(ctx)
        assert np.array_equal(got, O.oracle_gemm(A, B, wa, wb, sa, sb)), (case, wa, ea, wb, eb)
    assert _capi.load().gbs_debug_tc_error() == 0


def test_pair_auto_fills_the_gpu_for_few_tiles():
    """256 x 9216 x 4096 has 16 tiles of 256 x 256: the built-in rule narrows the tiles and/or
    splits K so that at least half of the SM pairs work, bit-exact."""
    import torch
    pairs = torch.cuda.get_device_properties(0).multi_processor_count // 2
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload("gemm_256x9216x4096_bpbp")
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    try:
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        assert sha(ctx.res.reshape(N, M)) == CFG["gemm_256x9216x4096_bpbp"]["sha256"]
        bn, sp = last_pair(ctx)
        assert bn in (128, 256) and sp >= 2 and (N // bn) * sp * 2 >= pairs, (bn, sp, pairs)
    finally:
        deallocGEMMContext(ctx)


PERSIST_CASES = [(512, 1024, 768), (300, 700, 600), (1024, 512, 1024), (257, 2048, 513)]


@pytest.mark.parametrize("shape", PERSIST_CASES, ids=[f"{m}x{k}x{n}" for (m, k, n) in PERSIST_CASES])
def test_pair_persistent(shape):
    """Persistent SM pairs (variant 514: ~3 tiles per pair, so both TMEM accumulators are reused)."""
    M, K, N = shape
    rng = np.random.default_rng(M + 3 * K + 5 * N)
    for (wa, ea, wb, eb) in [(3, "u", 2, "s"), (1, "b", 1, "b"), (4, "s", 1, "u"), (2, "s", 3, "u")]:
        A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
        sa, sb = ea != "u", eb != "u"
        ctx = allocGEMMContext(M, K, N, wa, wb, sa, sb)
        try:
            _capi.check(_capi.load().gbs_set_variant(ctx._h, 514))
            ctx.set_pipe(_capi.GBS_PIPE_TC)
            ctx.lhs.importRegular(A)
            ctx.rhs.importRegular(B)
            gemmBitSerial(ctx)
            got = ctx.res.reshape(N, M).copy()
            assert last_pair(ctx, True) == (256, 1, 1)
            gemmBitSerial(ctx)  # a second launch over the same context
            assert np.array_equal(ctx.res.reshape(N, M), got)
        finally:
            deallocGEMMContext(ctx)
        assert np.array_equal(got, O.oracle_gemm(A, B, wa, wb, sa, sb)), (shape, wa, ea, wb, eb)
    assert _capi.load().gbs_debug_tc_error() == 0


def test_pair_persistent_full_size():
    """4096 x 2048 x 2048 (128 tiles of 256 x 256, past one wave) on the persistent kernel: the
    reference's result bits."""
    name = "gemm_4096x2048x2048_u2bp"
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    try:
        _capi.check(_capi.load().gbs_set_variant(ctx._h, 514))
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        assert sha(ctx.res.reshape(N, M)) == CFG[name]["sha256"]
        assert last_pair(ctx, True) == (256, 1, 1)
    finally:
        deallocGEMMContext(ctx)


def test_pair_auto_goes_persistent_past_one_wave():
    """4096 x 2048 x 2048 has 128 tiles of 256 x 256, more than one wave: the built-in rule runs the
    persistent kernel, bit-exact."""
    name = "gemm_4096x2048x2048_u2bp"
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    try:
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        assert sha(ctx.res.reshape(N, M)) == CFG[name]["sha256"]
        assert last_pair(ctx, True) == (256, 1, 1)
    finally:
        deallocGEMMContext(ctx)


# stream-K shapes: tiles split over 2, 3 and 5 pairs, and an uneven split over every pair the GPU holds
STREAMK_CASES = [(300, 2000, 600), (700, 3000, 900), (257, 5000, 513), (1024, 8192, 1024)]


@pytest.mark.parametrize("shape", STREAMK_CASES, ids=[f"{m}x{k}x{n}" for (m, k, n) in STREAMK_CASES])
def test_pair_streamk(shape):
    """Stream-K SM pairs (variant 515): (tile, K stage) units split evenly over the pairs, split tiles
    finished by the pair holding their last stage from the lower pairs' fp32 partials; a second
    launch over the same context (the next epoch of the partials' flags) gives the same bits."""
    M, K, N = shape
    rng = np.random.default_rng(M + 7 * K + 11 * N)
    for (wa, ea, wb, eb) in [(3, "u", 2, "s"), (1, "b", 1, "b"), (4, "s", 1, "u")]:
        A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
        sa, sb = ea != "u", eb != "u"
        ctx = allocGEMMContext(M, K, N, wa, wb, sa, sb)
        try:
            _capi.check(_capi.load().gbs_set_variant(ctx._h, 515))
            ctx.set_pipe(_capi.GBS_PIPE_TC)
            ctx.lhs.importRegular(A)
            ctx.rhs.importRegular(B)
            gemmBitSerial(ctx)
            got = ctx.res.reshape(N, M).copy()
            bn, pairs, kind = last_pair(ctx, True)
            assert (bn, kind) == (256, 2) and pairs >= 1
            gemmBitSerial(ctx)
            assert np.array_equal(ctx.res.reshape(N, M), got)
        finally:
            deallocGEMMContext(ctx)
        assert np.array_equal(got, O.oracle_gemm(A, B, wa, wb, sa, sb, threads=8)), (shape, wa, ea, wb, eb)
    assert _capi.load().gbs_debug_tc_error() == 0


@pytest.mark.parametrize("name", ["gemm_2048x4096x2048_u3s2", "gemm_256x9216x4096_bpbp", "gemm_256x9216x4096_bps4",
                                  "gemm_4096x2048x2048_u2bp"])
def test_pair_streamk_full_size(name):
    """The full-size workloads on the stream-K kernel: the reference's result bits."""
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    try:
        _capi.check(_capi.load().gbs_set_variant(ctx._h, 515))
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        for _ in range(2):
            gemmBitSerial(ctx)
            assert sha(ctx.res.reshape(N, M)) == CFG[name]["sha256"]
        bn, pairs, kind = last_pair(ctx, True)
        assert (bn, kind) == (256, 2) and pairs >= 1
    finally:
        deallocGEMMContext(ctx)
    assert _capi.load().gbs_debug_tc_error() == 0


# explicit tile width x K split variants (a split that cannot run falls back to 1)
SPLIT_VARIANTS = [(2561, 256, 1), (2562, 256, 2), (2564, 256, 4), (1281, 128, 1), (1282, 128, 2), (1284, 128, 4)]


@pytest.mark.parametrize("case", SPLIT_VARIANTS, ids=[str(c[0]) for c in SPLIT_VARIANTS])
def test_pair_explicit_split_variants(case):
    variant, bn_want, split_want = case
    M, K, N = 512, 4096, 512
    rng = np.random.default_rng(variant)
    A = datagen.operand(int(rng.integers(1 << 30)), M, K, 3, "u")
    B = datagen.operand(int(rng.integers(1 << 30)), N, K, 2, "s")
    ctx = allocGEMMContext(M, K, N, 3, 2, False, True)
    try:
        _capi.check(_capi.load().gbs_set_variant(ctx._h, variant))
        ctx.set_pipe(_capi.GBS_PIPE_TC)
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        got = ctx.res.reshape(N, M).copy()
        assert last_pair(ctx, True) == (bn_want, split_want, 0)
    finally:
        deallocGEMMContext(ctx)
    assert np.array_equal(got, O.oracle_gemm(A, B, 3, 2, False, True))
