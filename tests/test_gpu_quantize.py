"""Threshold-quantising import (importRegularAndQuantize, gemmbitserial.hpp:282-305)
on the GPU: bit-exact against the reference's own results (tests/golden/ref_quantize.npz)
for every element type, column-major input, unsorted and empty threshold sets and
more levels than the bit width holds; then the GEMM that consumes the quantised
operand, on the CUDA-core and tensor-core pipes."""
import ctypes as C
import os

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def lib(gbs_lib):
    import torch
    assert torch.cuda.is_available()
    return gbs_lib


def cases():
    z = np.load(os.path.join(GOLD, "ref_quantize.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    return [(k, z[k + "_src"], z[k + "_thr"], z[k + "_meta"], z[k + "_values"]) for k in keys]


def export(ctx, side, rows, cols):
    out = np.zeros((rows, cols), np.int32)
    if rows * cols:
        _capi.check(_capi.load().gbs_export(ctx._h, side, C.c_void_p(out.ctypes.data), None))
    return out


@pytest.mark.parametrize("device", [False, True], ids=["host", "device"])
def test_quantize_matches_reference(device):
    import torch
    for key, src, thr, meta, want in cases():
        rows, cols, bits, nthres, cm = (int(x) for x in meta)
        ctx = allocGEMMContext(rows, cols, 1, bits, 1, False, False)
        try:
            s, t = (torch.from_numpy(src).cuda(), torch.from_numpy(thr).cuda()) if device else (src, thr)
            ctx.lhs.importRegularAndQuantize(s, t if nthres else None, nthres, readColMajor=bool(cm))
            torch.cuda.synchronize()
            assert np.array_equal(export(ctx, 0, rows, cols), want), key
        finally:
            deallocGEMMContext(ctx)


@pytest.mark.parametrize("pipe", [_capi.GBS_PIPE_AUTO, _capi.GBS_PIPE_POPC, _capi.GBS_PIPE_TC])
def test_gemm_after_quantized_import(pipe):
    """Activations quantised by per-channel thresholds, then the GEMM with signed weights."""
    rng = np.random.default_rng(7)
    for (M, K, N, bits, nthres, cm) in [(300, 640, 256, 2, 3, False), (96, 200, 70, 3, 7, True),
                                        (256, 1024, 512, 4, 15, False), (5, 64, 3, 2, 3, False)]:
        x = rng.normal(0, 2, (M, K)).astype(np.float32)
        thr = np.sort(rng.normal(0, 2, (nthres, M)).astype(np.float32), axis=0)
        src = np.ascontiguousarray(x.T) if cm else x
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, 3, "s")
        Aq = O.quantize_values(src, thr, bits, cm).astype(np.int8)
        want = O.oracle_gemm(Aq, B, bits, 3, False, True)
        ctx = allocGEMMContext(M, K, N, bits, 3, False, True)
        try:
            ctx.set_pipe(pipe)
            ctx.lhs.importRegularAndQuantize(src, thr, readColMajor=cm)
            ctx.rhs.importRegular(B)
            gemmBitSerial(ctx)
            assert np.array_equal(ctx.res.reshape(N, M), want), (M, K, N, bits, nthres, cm, ctx.pipe)
        finally:
            deallocGEMMContext(ctx)


def test_quantize_rejects_signed_and_bad_arguments(lib):
    ctx = allocGEMMContext(8, 64, 8, 2, 2, True, False)
    try:
        x = np.zeros((8, 64), np.float32)
        t = np.zeros((1, 8), np.float32)
        rc = lib.gbs_import_quantize(ctx._h, 0, C.c_void_p(x.ctypes.data), C.c_void_p(t.ctypes.data), 1,
                                     _capi.GBS_F32, 0, None)
        assert rc == _capi.GBS_EINVAL and b"unsigned" in lib.gbs_last_error()
        rc = lib.gbs_import_quantize(ctx._h, 1, C.c_void_p(x.ctypes.data), None, 2, _capi.GBS_F32, 0, None)
        assert rc == _capi.GBS_EINVAL  # thresholds missing
        rc = lib.gbs_import_quantize(ctx._h, 1, C.c_void_p(x.ctypes.data), None, -1, _capi.GBS_F32, 0, None)
        assert rc == _capi.GBS_EINVAL
        rc = lib.gbs_import_quantize(ctx._h, 1, C.c_void_p(x.ctypes.data), None, 0, 9, 0, None)
        assert rc == _capi.GBS_EINVAL
    finally:
        deallocGEMMContext(ctx)
