"""GPU parity: the CUDA path through the C ABI against the oracle and the
reference's golden vectors.  Every comparison is bit-exact.

These mirror the reference's own tests (test/test.cpp) through the Python
mirror of its API, then go beyond them: every encoding pair, col-major import,
wide element types, out-of-range values, odd shapes, empty shapes, full-size
workloads and both forward pipes.
"""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

import make_golden as G
from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import (allocGEMMContext, deallocGEMMContext, gemmBitSerial, sumRows)
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
VEC = json.load(open(os.path.join(GOLD, "ref_vectors.json")))
SMALL = np.load(os.path.join(GOLD, "ref_results_small.npz"))
CFG = json.load(open(os.path.join(GOLD, "ref_configs.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module", autouse=True)
def lib(gbs_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return gbs_lib


def gpu_gemm(A, B, wA, wB, sA, sB, cmA=False, cmB=False, pipe=None):
    M, K = (A.shape[1], A.shape[0]) if cmA else A.shape
    N = B.shape[1] if cmB else B.shape[0]
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    try:
        if pipe is not None:
            ctx.set_pipe(pipe)
        ctx.lhs.importRegular(A, cmA)
        ctx.rhs.importRegular(B, cmB)
        gemmBitSerial(ctx)
        return ctx.res.reshape(N, M)
    finally:
        deallocGEMMContext(ctx)


PIPES = [_capi.GBS_PIPE_AUTO, _capi.GBS_PIPE_POPC, _capi.GBS_PIPE_BMMA, _capi.GBS_PIPE_TC, _capi.GBS_PIPE_TC_PAIRS,
         _capi.GBS_PIPE_TC_SMEM]


@pytest.mark.parametrize("c", VEC["gemm"], ids=[c["name"] for c in VEC["gemm"]])
def test_reference_vectors(c):
    """The reference's test grids (test/test.cpp:110-277) and the extra mixed grid."""
    A = G.operand(c["seed"], c["M"], c["K"], c["wA"], c["sA"], c["dtA"], c["kind"])
    B = G.operand(c["seed"] + 1, c["N"], c["K"], c["wB"], c["sB"], c["dtB"], c["kind"])
    Ain = np.ascontiguousarray(A.T) if c["cmA"] else A
    Bin = np.ascontiguousarray(B.T) if c["cmB"] else B
    res = gpu_gemm(Ain, Bin, c["wA"], c["wB"], c["sA"], c["sB"], bool(c["cmA"]), bool(c["cmB"]))
    assert sha(res) == c["sha_res"]
    if c["name"] in SMALL.files:
        assert np.array_equal(res, SMALL[c["name"]])


def test_mnist_known_answer():
    z = np.load(os.path.join(GOLD, "mnist_kat.npz"))
    n_out, n_in = [int(v) for v in z["shape"]]
    w = np.unpackbits(z["w_bits"])[: n_out * n_in].reshape(n_out, n_in).astype(np.int8) * 2 - 1
    wb, ab, ws, as_ = [int(v) for v in z["flags"]]
    for pipe in PIPES:
        res = gpu_gemm(w, z["x"].reshape(1, -1), wb, ab, ws, as_, pipe=pipe)
        assert np.array_equal(res.ravel(), z["golden"])


@pytest.mark.parametrize("r", VEC["rows"], ids=[f"b{r['b']}_d{r['d']}_s{r['s']}" for r in VEC["rows"]])
def test_rowsums_and_export(r):
    """test/test.cpp:30-108: sumRows and import -> exportRegular, compared in full."""
    X = G.operand(r["seed"], r["d"], r["d"], r["b"], r["s"], "i8", "in")
    ctx = allocGEMMContext(r["d"], r["d"], 1, r["b"], 1, r["s"], 0)
    try:
        ctx.lhs.importRegular(X)
        assert [int(v) for v in sumRows(ctx.lhs)] == r["sum"]
        assert sha(ctx.lhs.exportRegular().astype(np.int32)) == r["sha_export"]
    finally:
        deallocGEMMContext(ctx)


def test_packed_planes_match_oracle():
    """Device planes hold the reference layout with the reference's padding."""
    rng = np.random.default_rng(5)
    for dt in (np.int8, np.uint8, np.int16, np.int32):
        for cm in (False, True):
            for (M, K, bits, sgn) in [(37, 300, 3, 1), (128, 4096, 2, 0), (5, 64, 1, 1), (200, 777, 8, 0)]:
                X = rng.integers(-100, 100, (M, K)).astype(dt) if dt != np.uint8 else rng.integers(0, 256, (M, K)).astype(dt)
                Xin = np.ascontiguousarray(X.T) if cm else X
                ctx = allocGEMMContext(M, K, 3, bits, 1, sgn, 0)
                oc = O.OracleContext(M, K, 3, bits, 1, sgn, 0)
                try:
                    ctx.lhs.importRegular(Xin, cm)
                    oc.import_(0, Xin, cm)
                    dev = ctx.lhs.planes()
                    ref = oc.planes(0)
                    # the reference's geometry and padding, word for word (padding zero in both)
                    assert dev.shape == ref.shape, (dt, cm, M, K)
                    assert np.array_equal(dev, ref), (dt, cm, M, K)
                finally:
                    deallocGEMMContext(ctx)
                    oc.close()


ENCS = [(1, "u"), (1, "b"), (2, "u"), (2, "s"), (3, "u"), (3, "s"), (4, "s"), (8, "u"), (8, "s")]


@pytest.mark.parametrize("pipe", PIPES)
def test_every_encoding_pair(pipe):
    rng = np.random.default_rng(17)
    for (wa, ea) in ENCS:
        for (wb, eb) in ENCS:
            M, K, N = int(rng.integers(60, 150)), int(rng.integers(60, 900)), int(rng.integers(60, 150))
            A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
            B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
            sa, sb = ea != "u", eb != "u"
            ref = O.oracle_gemm(A, B, wa, wb, sa, sb)
            assert np.array_equal(gpu_gemm(A, B, wa, wb, sa, sb, pipe=pipe), ref), (wa, ea, wb, eb)


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 64, 1), (3, 1, 5), (128, 256, 128), (129, 257, 130),
                                   (16, 64, 4000), (4000, 64, 16), (64, 9000, 64), (300, 4096, 1),
                                   (1, 4096, 300), (2, 8192, 2), (255, 63, 257)])
def test_odd_and_skinny_shapes(shape):
    M, K, N = shape
    rng = np.random.default_rng(M * 7 + K * 3 + N)
    for (wa, ea, wb, eb) in [(1, "u", 1, "u"), (3, "u", 2, "s"), (1, "b", 1, "b"), (1, "b", 4, "s"), (2, "u", 1, "b")]:
        A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
        sa, sb = ea != "u", eb != "u"
        ref = O.oracle_gemm(A, B, wa, wb, sa, sb)
        for pipe in PIPES:
            assert np.array_equal(gpu_gemm(A, B, wa, wb, sa, sb, pipe=pipe), ref), (shape, wa, ea, wb, eb, pipe)


@pytest.mark.parametrize("M", [1, 2, 3, 4, 5, 6, 8, 9, 12, 13, 16])
def test_popc_rows_tile(lib, M):
    """The CUDA cores' rows tile (at most 16 lhs rows x 64-256 rhs rows, 1-4 threads per rhs row), forced
    (variant 4) and by the built-in rule: every M bucket, odd and even words per row, rhs row counts
    off the tile, bipolar x bipolar (XOR), bipolar x regular (row sums), signed, 8-bit planes."""
    rng = np.random.default_rng(100 + M)
    for (K, N) in [(64 * 37 + 5, 700), (64 * 40, 256), (1000, 513)]:
        for (wa, ea, wb, eb) in [(1, "u", 1, "u"), (1, "b", 1, "b"), (1, "b", 4, "s"), (3, "s", 2, "u"),
                                 (8, "s", 3, "u"), (2, "u", 8, "s"), (4, "u", 1, "b")]:
            A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
            B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
            sa, sb = ea != "u", eb != "u"
            ref = O.oracle_gemm(A, B, wa, wb, sa, sb)
            for variant in (-1, 4):
                ctx = allocGEMMContext(M, K, N, wa, wb, sa, sb)
                try:
                    ctx.set_pipe(_capi.GBS_PIPE_POPC)
                    _capi.check(lib.gbs_set_variant(ctx._h, variant))
                    ctx.lhs.importRegular(A)
                    ctx.rhs.importRegular(B)
                    gemmBitSerial(ctx)
                    got = ctx.res.reshape(N, M)
                finally:
                    deallocGEMMContext(ctx)
                assert np.array_equal(got, ref), (M, K, N, wa, ea, wb, eb, variant)


def test_empty_shapes():
    for (M, K, N) in [(0, 64, 5), (5, 64, 0), (0, 0, 0)]:
        ctx = allocGEMMContext(M, K, N, 2, 2, 0, 0)
        ctx.lhs.importRegular(np.zeros((M, K), np.int8))
        ctx.rhs.importRegular(np.zeros((N, K), np.int8))
        gemmBitSerial(ctx)
        assert ctx.res.size == 0
        deallocGEMMContext(ctx)
    # K == 0: every product is an empty sum; bipolar x bipolar gives ncols = 0 too
    for (wa, sa, wb, sb) in [(2, 0, 2, 0), (1, 1, 1, 1), (1, 1, 3, 1)]:
        res = gpu_gemm(np.zeros((4, 0), np.int8), np.zeros((3, 0), np.int8), wa, wb, sa, sb)
        assert np.array_equal(res, O.oracle_gemm(np.zeros((4, 0), np.int8), np.zeros((3, 0), np.int8), wa, wb, sa, sb))


def test_int32_wraparound_matches_reference():
    """8-bit x 8-bit at large K overflows int32 in the reference; the GPU wraps identically."""
    M, K, N = 64, 140000, 64
    A = np.full((M, K), -128, np.int8)
    B = np.full((N, K), -128, np.int8)
    ref = O.oracle_gemm(A, B, 8, 8, 1, 1)
    assert np.array_equal(gpu_gemm(A, B, 8, 8, 1, 1), ref)
    assert (ref.astype(np.int64) != 128 * 128 * K).all()  # the case really wraps


@pytest.mark.parametrize("name", sorted(CFG))
def test_full_size_workloads(name):
    """Full-size benchmark workloads, bit-exact (sha256) against the reference's own results."""
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
    for pipe in PIPES:
        assert sha(gpu_gemm(A, B, wA, wB, sA, sB, pipe=pipe)) == CFG[name]["sha256"], pipe


def test_device_inputs_and_stream():
    import torch
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload("gemm_256x9216x4096_bps4")
    s = torch.cuda.Stream()
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    try:
        with torch.cuda.stream(s):
            ctx.lhs.importRegular(torch.from_numpy(A).cuda(), stream=s)
            ctx.rhs.importRegular(torch.from_numpy(B).cuda(), stream=s)
            gemmBitSerial(ctx, stream=s)
        s.synchronize()
        assert sha(ctx.res.reshape(N, M)) == CFG["gemm_256x9216x4096_bps4"]["sha256"]
    finally:
        deallocGEMMContext(ctx)


def test_repeated_gemm_is_idempotent():
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload("gemm_2048x4096x2048_u3s2")
    ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
    ctx.lhs.importRegular(A)
    ctx.rhs.importRegular(B)
    gemmBitSerial(ctx)
    r1 = ctx.res.copy()
    gemmBitSerial(ctx)
    gemmBitSerial(ctx)
    assert np.array_equal(ctx.res, r1)
    deallocGEMMContext(ctx)


def test_error_paths(lib):
    ctx = allocGEMMContext(8, 64, 8, 2, 2, 0, 0)
    with pytest.raises(_capi.GBSError) as e:
        gemmBitSerial(ctx)  # no import yet
    assert e.value.code == _capi.GBS_ESTATE
    with pytest.raises(TypeError):  # float32 is accepted (importRegular<float>); float64 is not
        ctx.lhs.importRegular(np.zeros((8, 64), np.float64))
    deallocGEMMContext(ctx)
    # host-side allocation failure injection: reported, nothing leaks, library stays usable
    for n in (1, 2, 3, 4):
        lib.gbs_debug_fail_alloc_after(n)
        h = C.c_void_p()
        rc = lib.gbs_ctx_alloc(100, 300, 100, 2, 2, 0, 0, C.byref(h))
        assert rc == _capi.GBS_ENOMEM and not h.value
    lib.gbs_debug_fail_alloc_after(0)
    A = np.ones((9, 70), np.int8)
    assert np.array_equal(gpu_gemm(A, A, 1, 1, 0, 0), np.full((9, 9), 70, np.int32))


def test_launches_are_counted(lib):
    before = lib.gbs_debug_launch_count()
    gpu_gemm(np.ones((4, 64), np.int8), np.ones((4, 64), np.int8), 1, 1, 0, 0)
    assert lib.gbs_debug_launch_count() >= before + 3  # two packs and one forward kernel


def test_context_geometry_is_the_references():
    """Every golden vector's context reports the reference's nrows_a, ncols_a, lhsBlock and rhsBlock
    (arch-generic.hpp:78-100, gemmbitserial.hpp:415-452), as recorded by the compiled reference."""
    from gemmbitserial_gb300 import _capi
    lib = _capi.load()
    seen = set()
    for v in VEC["gemm"]:
        key = (v["M"], v["K"], v["N"])
        if key in seen:
            continue
        seen.add(key)
        ctx = allocGEMMContext(v["M"], v["K"], v["N"], v["wA"], v["wB"], v["sA"], v["sB"])
        try:
            info = _capi.CtxInfo()
            _capi.check(lib.gbs_ctx_get_info(ctx._h, C.byref(info)))
            got = [info.lhs.nrows_a, info.rhs.nrows_a, info.lhs.ncols_a, info.rhs.ncols_a, info.lhsBlock, info.rhsBlock]
            assert got == v["ref_dims"], key
            assert ctx.lhs.planes().shape == (v["wA"], v["ref_dims"][0], v["ref_dims"][2] // 64)
        finally:
            deallocGEMMContext(ctx)
