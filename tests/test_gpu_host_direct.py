"""Host memory the device addresses directly: imports that pack a host source in
place (no staging copy) and gbs_gemm_to, whose kernels write the result into the
caller's buffer -- the fused gemmBitSerial + ctx.res read of the reference's
callers (arch-generic.hpp:331-345, gemmbitserial.hpp:383).  Both must give the
same bits as the staged path (GBS_HOST_DIRECT=0) and as gbs_gemm +
gbs_get_result, on every forward kernel family."""
import ctypes as C

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib(gbs_lib):
    import torch
    assert torch.cuda.is_available()
    return gbs_lib


@pytest.fixture
def staged(monkeypatch):
    monkeypatch.setenv("GBS_HOST_DIRECT", "0")


def planes(ctx, side):
    info = ctx._info()
    m = info.lhs if side == 0 else info.rhs
    out = np.zeros(max(m.nbits * m.nrows_a * (m.ncols_a // 64), 1), np.uint64)
    _capi.check(_capi.load().gbs_get_planes(ctx._h, side, C.c_void_p(out.ctypes.data), None))
    return out


# (M, K, N, wA, sA, wB, sB, pipe): the SM-pair kernel, its split-K form, the
# persistent one-problem kernel (a side under 256), the CUDA-core and BMMA pipes
SHAPES = [
    (512, 1024, 768, 3, False, 2, True, _capi.GBS_PIPE_AUTO),
    (256, 4096, 2304, 1, True, 1, True, _capi.GBS_PIPE_AUTO),
    (96, 640, 1000, 2, False, 2, True, _capi.GBS_PIPE_AUTO),
    (300, 700, 130, 2, True, 3, False, _capi.GBS_PIPE_POPC),
    (200, 512, 96, 1, False, 1, False, _capi.GBS_PIPE_BMMA),
]


def enc(w, signed):
    return "b" if (w == 1 and signed) else ("s" if signed else "u")


def make(M, K, N, wA, sA, wB, sB, seed):
    return (datagen.operand(seed, M, K, wA, enc(wA, sA)), datagen.operand(seed + 1, N, K, wB, enc(wB, sB)))


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{s[0]}x{s[1]}x{s[2]}p{s[7]}" for s in SHAPES])
def test_gemm_to_equals_gemm(shape):
    import torch
    M, K, N, wA, sA, wB, sB, pipe = shape
    A, B = make(M, K, N, wA, sA, wB, sB, datagen.SEED_BASE + 2000 + M)
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    try:
        ctx.set_pipe(pipe)
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        gemmBitSerial(ctx)
        want = ctx.res.copy()
        outs = {
            "pageable": np.full(M * N, -7, np.int32),
            "pinned": torch.full((M * N,), -7, dtype=torch.int32).pin_memory(),
            "device": torch.full((M * N,), -7, dtype=torch.int32, device="cuda"),
        }
        for name, out in outs.items():
            gemmBitSerial(ctx, out=out)
            torch.cuda.synchronize()
            got = out.cpu().numpy() if hasattr(out, "cpu") else out
            assert np.array_equal(got, want), (name, ctx.pipe)
        # a buffer off the 16-byte grid takes the compute-then-copy path
        raw = np.full(M * N + 1, -7, np.int32)
        gemmBitSerial(ctx, out=raw[1:])
        assert np.array_equal(raw[1:], want) and raw[0] == -7
    finally:
        deallocGEMMContext(ctx)


def test_gemm_to_matches_oracle():
    M, K, N = 300, 1000, 260
    A = datagen.operand(datagen.SEED_BASE + 2100, M, K, 3, "u")
    B = datagen.operand(datagen.SEED_BASE + 2101, N, K, 2, "s")
    ctx = allocGEMMContext(M, K, N, 3, 2, False, True)
    try:
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        out = np.zeros(M * N, np.int32)
        gemmBitSerial(ctx, out=out)
        assert np.array_equal(out.reshape(N, M), O.oracle_gemm(A, B, 3, 2, False, True))
    finally:
        deallocGEMMContext(ctx)


def test_result_stale_after_gemm_to(lib):
    """A direct write (pinned destination) leaves ctx.res stale; a pageable one is copied from it."""
    import torch
    M, K, N = 64, 256, 80
    ctx = allocGEMMContext(M, K, N, 2, 2, False, False)
    try:
        ctx.lhs.importRegular(datagen.operand(datagen.SEED_BASE + 2200, M, K, 2, "u"))
        ctx.rhs.importRegular(datagen.operand(datagen.SEED_BASE + 2201, N, K, 2, "u"))
        out = torch.zeros(M * N, dtype=torch.int32).pin_memory()
        gemmBitSerial(ctx, out=out)
        dst = np.zeros(M * N, np.int32)
        assert lib.gbs_get_result(ctx._h, C.c_void_p(dst.ctypes.data), None) == _capi.GBS_ESTATE
        assert b"gbs_gemm_to" in lib.gbs_last_error()
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res, out.numpy())
        page = np.zeros(M * N, np.int32)
        gemmBitSerial(ctx, out=page)
        assert np.array_equal(ctx.res, page)  # still valid: computed into res, then copied
        assert lib.gbs_gemm_to(ctx._h, None, None) == _capi.GBS_EINVAL
    finally:
        deallocGEMMContext(ctx)


@pytest.mark.parametrize("src_kind", ["pageable", "pinned"])
@pytest.mark.parametrize("col_major", [False, True], ids=["rows", "cols"])
def test_direct_import_equals_staged(src_kind, col_major, monkeypatch):
    """Same planes and GEMM from a host source packed in place and from the staged copies."""
    import torch
    M, K, N = 300, 2000, 260
    rng = np.random.default_rng(5)
    cases = [(np.int8, 3, False), (np.float32, 2, True), (np.int16, 4, True)]
    for dt, bits, sgn in cases:
        lo, hi = (-(1 << (bits - 1)), 1 << (bits - 1)) if sgn else (0, 1 << bits)
        A = rng.integers(lo, hi, (M, K)).astype(dt)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, 2, "s")
        src = np.ascontiguousarray(A.T) if col_major else A
        if src_kind == "pinned":
            src = torch.from_numpy(src).pin_memory()
        results, plane_sets = [], []
        for direct in ("1", "0"):
            monkeypatch.setenv("GBS_HOST_DIRECT", direct)
            ctx = allocGEMMContext(M, K, N, bits, 2, sgn, True)
            try:
                ctx.lhs.importRegular(src, readColMajor=col_major)
                ctx.rhs.importRegular(B)
                gemmBitSerial(ctx)
                results.append(ctx.res.copy())
                plane_sets.append(planes(ctx, 0))
            finally:
                deallocGEMMContext(ctx)
        assert np.array_equal(plane_sets[0], plane_sets[1]), (dt, src_kind, col_major)
        assert np.array_equal(results[0], results[1]), (dt, src_kind, col_major)
        want = O.oracle_gemm(A.astype(np.int64).astype(np.int8), B, bits, 2, sgn, True)
        assert np.array_equal(results[0].reshape(N, M), want), (dt, src_kind, col_major)


def test_staged_import_still_exact(staged):
    M, K, N = 256, 1536, 512
    A = datagen.operand(datagen.SEED_BASE + 2300, M, K, 2, "u")
    B = datagen.operand(datagen.SEED_BASE + 2301, N, K, 3, "s")
    ctx = allocGEMMContext(M, K, N, 2, 3, False, True)
    try:
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        out = np.zeros(M * N, np.int32)
        gemmBitSerial(ctx, out=out)  # staged everywhere: compute into res, then copy
        assert np.array_equal(out.reshape(N, M), O.oracle_gemm(A, B, 2, 3, False, True))
    finally:
        deallocGEMMContext(ctx)


def test_staged_host_import_mode(lib):
    """gbs_set_host_import(GBS_HOST_IMPORT_STAGED): host sources (pinned and pageable) go through the
    copy-engine staging path of this context only; same planes and results as reading in place, and
    as the oracle; unknown modes are refused."""
    import torch
    M, K, N = 300, 1000, 260
    A = datagen.operand(datagen.SEED_BASE + 2300, M, K, 3, "u")
    B = datagen.operand(datagen.SEED_BASE + 2301, N, K, 2, "s")
    want = O.oracle_gemm(A, B, 3, 2, False, True)
    got = {}
    for mode in (_capi.GBS_HOST_IMPORT_AUTO, _capi.GBS_HOST_IMPORT_STAGED):
        for kind in ("pageable", "pinned"):
            ctx = allocGEMMContext(M, K, N, 3, 2, False, True)
            try:
                ctx.set_host_import(mode)
                a = A if kind == "pageable" else torch.from_numpy(A).pin_memory()
                b = B if kind == "pageable" else torch.from_numpy(B).pin_memory()
                ctx.lhs.importRegular(a)
                ctx.rhs.importRegular(b)
                gemmBitSerial(ctx)
                assert np.array_equal(ctx.res.reshape(N, M), want), (mode, kind)
                got[(mode, kind)] = (planes(ctx, 0), planes(ctx, 1))
            finally:
                deallocGEMMContext(ctx)
    ref = got[(_capi.GBS_HOST_IMPORT_AUTO, "pageable")]
    for key, (pl, pr) in got.items():
        assert np.array_equal(pl, ref[0]) and np.array_equal(pr, ref[1]), key
    ctx = allocGEMMContext(8, 64, 8, 1, 1, False, False)
    try:
        assert lib.gbs_set_host_import(ctx._h, 2) == _capi.GBS_EINVAL
        assert lib.gbs_set_host_import(None, 0) == _capi.GBS_EINVAL
    finally:
        deallocGEMMContext(ctx)
