"""gbs_tune: times every applicable pipe/variant on a context's own data,
records the winner for its shape class, and the automatic choice follows it;
results stay bit-exact whatever the choice."""
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


def test_tune_records_winner_and_stays_exact(gbs_lib, tmp_path):
    lib = gbs_lib
    lib.gbs_tuner_clear()
    cfg = json.load(open(os.path.join(GOLD, "ref_configs.json")))
    for name in ["gemm_2048x4096x2048_u3s2", "gemm_256x9216x4096_bpbp"]:
        M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
        ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        best = C.c_int()
        _capi.check(lib.gbs_tune(ctx._h, 3, C.byref(best), None))
        assert best.value in (_capi.GBS_PIPE_POPC, _capi.GBS_PIPE_BMMA, _capi.GBS_PIPE_TC, _capi.GBS_PIPE_TC_PAIRS,
                              _capi.GBS_PIPE_TC_SMEM)
        assert ctx.pipe == best.value  # AUTO follows the store
        gemmBitSerial(ctx)
        got = ctx.res.reshape(N, M)
        assert hashlib.sha256(np.ascontiguousarray(got).tobytes()).hexdigest() == cfg[name]["sha256"]
        deallocGEMMContext(ctx)
    assert lib.gbs_tuner_entries() == 2
    path = str(tmp_path / "store.txt").encode()
    _capi.check(lib.gbs_tuner_save(path))
    lib.gbs_tuner_clear()
    _capi.check(lib.gbs_tuner_load(path, 1))
    assert lib.gbs_tuner_entries() == 2
    lib.gbs_tuner_clear()


CANDIDATES = [(_capi.GBS_PIPE_POPC, v) for v in (-1, 0, 1, 2)] + [(_capi.GBS_PIPE_BMMA, -1)] + \
    [(_capi.GBS_PIPE_TC, 128), (_capi.GBS_PIPE_TC, 256), (_capi.GBS_PIPE_TC_SMEM, 128), (_capi.GBS_PIPE_TC_SMEM, 256),
     (_capi.GBS_PIPE_TC_PAIRS, 128), (_capi.GBS_PIPE_TC_PAIRS, 256)] + \
    [(_capi.GBS_PIPE_TC, v) for v in (-1, 512, 513, 514, 515, 2561, 2562, 2564, 1281, 1282, 1284)]


def test_every_candidate_is_exact(gbs_lib):
    """Every (pipe, variant) the tuner may pick gives the oracle's result."""
    lib = gbs_lib
    rng = np.random.default_rng(8)
    for (M, K, N, wa, ea, wb, eb) in [(300, 1000, 500, 3, "u", 2, "s"), (130, 640, 260, 1, "b", 1, "b")]:
        A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
        want = O.oracle_gemm(A, B, wa, wb, ea != "u", eb != "u")
        ctx = allocGEMMContext(M, K, N, wa, wb, ea != "u", eb != "u")
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        for pipe, var in CANDIDATES:
            _capi.check(lib.gbs_set_pipe(ctx._h, pipe))
            _capi.check(lib.gbs_set_variant(ctx._h, var))
            gemmBitSerial(ctx)
            assert np.array_equal(ctx.res.reshape(N, M), want), (M, K, N, pipe, var)
        deallocGEMMContext(ctx)


def test_tuned_variants_are_exact(gbs_lib):
    """The tuner's pick gives the oracle's result."""
    lib = gbs_lib
    rng = np.random.default_rng(9)
    for (M, K, N, wa, ea, wb, eb) in [(300, 1000, 500, 3, "u", 2, "s"), (40, 2000, 700, 1, "b", 4, "s"),
                                      (130, 640, 260, 2, "s", 2, "u")]:
        A = datagen.operand(int(rng.integers(1 << 30)), M, K, wa, ea)
        B = datagen.operand(int(rng.integers(1 << 30)), N, K, wb, eb)
        want = O.oracle_gemm(A, B, wa, wb, ea != "u", eb != "u")
        ctx = allocGEMMContext(M, K, N, wa, wb, ea != "u", eb != "u")
        ctx.lhs.importRegular(A)
        ctx.rhs.importRegular(B)
        best = C.c_int()
        _capi.check(lib.gbs_tune(ctx._h, 1, C.byref(best), None))
        gemmBitSerial(ctx)
        assert np.array_equal(ctx.res.reshape(N, M), want), (M, K, N, best.value)
        deallocGEMMContext(ctx)
    lib.gbs_tuner_clear()


def test_committed_store_covers_the_workloads_and_stays_exact(gbs_lib):
    """The GB300 tuner store committed with the library (gemmbitserial_gb300/tuned, written by
    gemmbitserial_gb300.tune_workloads) has an entry for every named workload, and the kernels it
    picks give the reference's result bits."""
    lib = gbs_lib
    store = os.path.join(os.path.dirname(GOLD), "..", "gemmbitserial_gb300", "tuned", "gb300_sm103a.txt")
    _capi.check(lib.gbs_tuner_load(os.path.abspath(store).encode(), 1))
    cfg = json.load(open(os.path.join(GOLD, "ref_configs.json")))
    try:
        for name in datagen.WORKLOADS:
            M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
            ctx = allocGEMMContext(M, K, N, wA, wB, sA, sB)
            try:
                pipe, var, us = C.c_int(), C.c_int(), C.c_double()
                _capi.check(lib.gbs_tuner_lookup(ctx._h, C.byref(pipe), C.byref(var), C.byref(us)))
                assert ctx.pipe == pipe.value and us.value > 0, name
                ctx.lhs.importRegular(A)
                ctx.rhs.importRegular(B)
                gemmBitSerial(ctx)
                got = ctx.res.reshape(N, M)
                assert hashlib.sha256(np.ascontiguousarray(got).tobytes()).hexdigest() == cfg[name]["sha256"], name
            finally:
                deallocGEMMContext(ctx)
    finally:
        lib.gbs_tuner_clear()
