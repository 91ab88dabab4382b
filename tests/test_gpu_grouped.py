"""Grouped GEMM (one persistent launch over many contexts, optionally captured
with the packing into a CUDA graph): bit-exact per problem against the oracle
on a reduced mix, and on the full 512-problem mix against both the oracle and
the plain per-problem GPU path."""
import os

import numpy as np
import pytest

from gemmbitserial_gb300 import _capi, datagen
from gemmbitserial_gb300.api import allocGEMMContext, deallocGEMMContext, gemmBitSerial
from gemmbitserial_gb300.grouped import Group
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def lib(gbs_lib):
    import torch
    assert torch.cuda.is_available()
    return gbs_lib


def make_contexts(mix):
    return [allocGEMMContext(M, K, N, wA, wB, eA != "u", eB != "u") for (M, K, N, wA, eA, wB, eB) in mix]


@pytest.fixture(params=["auto", "tc", "tc-digits", "tc-nibbles", "popc"])
def group_pipe(request, monkeypatch):
    """GBS_GROUP_PIPE as read by gbs_group_create: per-problem choice, or one kernel forced;
    tc-digits / tc-nibbles also force the tensor-core problems' kernel (GBS_TCG_NIBBLES=0 / 1)
    where plain tc leaves it to the library's estimate."""
    monkeypatch.delenv("GBS_TCG_NIBBLES", raising=False)
    if request.param == "auto":
        monkeypatch.delenv("GBS_GROUP_PIPE", raising=False)
    else:
        monkeypatch.setenv("GBS_GROUP_PIPE", request.param.split("-")[0])
    if request.param == "tc-digits":
        monkeypatch.setenv("GBS_TCG_NIBBLES", "0")
    if request.param == "tc-nibbles":
        monkeypatch.setenv("GBS_TCG_NIBBLES", "1")
    return request.param


def check_split(g, mode, count):
    st = g.stats()
    assert st["popc_problems"] + st["tc_problems"] == count
    if mode == "popc":
        assert st["tc_problems"] == 0
        assert st["tc_kernel"] == "none"
    if mode.startswith("tc"):
        assert st["tc_problems"] > 0
        want = {"tc-digits": ("digits",), "tc-nibbles": ("nibbles",)}.get(mode, ("digits", "nibbles"))
        assert st["tc_kernel"] in want
    return st


def test_grouped_reduced_mix_matches_oracle(group_pipe):
    import torch
    mix = datagen.grouped_mix(seed=datagen.SEED_BASE + 77, count=96, k_words=(1, 40), n_range=(1, 700))
    host = []
    for i, (M, K, N, wA, eA, wB, eB) in enumerate(mix):
        A = datagen.operand(datagen.SEED_BASE + 1000 + 2 * i, M, K, wA, eA)
        B = datagen.operand(datagen.SEED_BASE + 1001 + 2 * i, N, K, wB, eB)
        if i % 5 == 1:  # exercise other element types through the grouped pack
            A = A.astype(np.int32)
        if i % 7 == 2 and eB != "b":
            B = (B.astype(np.int16) & 0xFF).astype(np.uint8) if eB == "u" else B.astype(np.int16)
        host.append((A, B))
    ctxs = make_contexts(mix)
    dev = [(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()) for A, B in host]
    s = torch.cuda.Stream()
    g = Group(ctxs)
    try:
        check_split(g, group_pipe, len(mix))
        with torch.cuda.stream(s):
            g.import_([a for a, _ in dev], [b for _, b in dev], stream=s)
            g.gemm(stream=s)
        s.synchronize()
        assert g.status(s) == _capi.GBS_OK
        for (M, K, N, wA, eA, wB, eB), (A, B), c in zip(mix, host, ctxs):
            want = O.oracle_gemm(A, B, wA, wB, eA != "u", eB != "u")
            assert np.array_equal(c.res.reshape(N, M), want), (M, K, N, wA, eA, wB, eB)
        # the captured graph (pack + gemm) reproduces it, twice in a row
        with torch.cuda.stream(s):
            g.capture([a for a, _ in dev], [b for _, b in dev], stream=s)
            g.replay(stream=s)
            g.replay(stream=s)
        s.synchronize()
        for (M, K, N, wA, eA, wB, eB), (A, B), c in zip(mix, host, ctxs):
            want = O.oracle_gemm(A, B, wA, wB, eA != "u", eB != "u")
            assert np.array_equal(c.res.reshape(N, M), want)
    finally:
        g.free()
        for c in ctxs:
            deallocGEMMContext(c)


# Tile geometry of the tensor-core kernel: lhs-major and rhs-major problems,
# MMA N from 16 to 256, several column tiles, M not a multiple of 4, 1-row
# operands, K not a multiple of 128, every encoding pair, and the largest K
# whose sums stay exact in fp32 for 4 x 4-bit unsigned operands.
EDGE_MIX = [
    (300, 640, 70, 2, "u", 3, "s"),      # M > N: lhs is the MMA row operand
    (520, 1000, 600, 1, "b", 2, "u"),    # M < N, both > 256: 3 column tiles of 256
    (17, 333, 129, 4, "s", 1, "b"),      # M odd: scalar stores of result rows
    (1, 64, 1, 1, "u", 1, "u"),
    (1, 4096, 3000, 4, "u", 4, "s"),
    (256, 192, 256, 1, "b", 1, "b"),
    (128, 2048, 128, 3, "u", 3, "u"),
    (64, 74565, 96, 4, "u", 4, "u"),     # 74565 * 15 * 15 < 2^24
    (96, 512, 48, 2, "s", 4, "s"),
    (200, 129, 1, 2, "u", 2, "u"),
    # the nibble kernel's larger operand of every width and encoding, odd words per
    # row, several 256-row column tiles, and K at the fp32 exactness limit
    (333, 960, 40, 3, "s", 2, "u"),      # wpr 15
    (5, 1088, 777, 1, "u", 3, "s"),      # wpr 17
    (9, 1472, 391, 2, "u", 1, "b"),      # wpr 23, bipolar row operand
    (41, 4992, 300, 3, "u", 1, "u"),
    (40, 74560, 130, 4, "u", 3, "u"),    # wpr 1165
    (40, 80000, 130, 4, "u", 3, "u"),    # 80000 * 15 * 7 < 2^24
    # few lhs rows: the CUDA cores' rows tile when the built-in rule keeps them there
    (3, 1000, 700, 1, "b", 1, "b"),      # XOR, wpr 16
    (9, 64 * 37 + 5, 513, 1, "u", 1, "u"),  # wpr 38, 3 tiles of 256 rhs rows
    (2, 4096, 3000, 2, "s", 2, "u"),
]


def test_grouped_tc_edge_shapes(group_pipe):
    import torch
    host = [(datagen.operand(datagen.SEED_BASE + 3000 + 2 * i, M, K, wA, eA),
             datagen.operand(datagen.SEED_BASE + 3001 + 2 * i, N, K, wB, eB))
            for i, (M, K, N, wA, eA, wB, eB) in enumerate(EDGE_MIX)]
    ctxs = make_contexts(EDGE_MIX)
    dev = [(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()) for A, B in host]
    g = Group(ctxs)
    try:
        st = check_split(g, group_pipe, len(EDGE_MIX))
        if group_pipe.startswith("tc"):
            assert st["tc_problems"] == len(EDGE_MIX)
        g.import_([a for a, _ in dev], [b for _, b in dev])
        g.gemm()
        torch.cuda.synchronize()
        assert g.status() == _capi.GBS_OK
        for (M, K, N, wA, eA, wB, eB), (A, B), c in zip(EDGE_MIX, host, ctxs):
            want = O.oracle_gemm(A, B, wA, wB, eA != "u", eB != "u", threads=8)
            assert np.array_equal(c.res.reshape(N, M), want), (M, K, N, wA, eA, wB, eB)
        # re-importing one context alone makes its digits stale; the group rebuilds them
        A2 = datagen.operand(datagen.SEED_BASE + 3999, 300, 640, 2, "u")
        ctxs[0].lhs.importRegular(torch.from_numpy(A2).cuda())
        g.gemm()
        torch.cuda.synchronize()
        want = O.oracle_gemm(A2, host[0][1], 2, 3, False, True)
        assert np.array_equal(ctxs[0].res.reshape(70, 300), want)
    finally:
        g.free()
        for c in ctxs:
            deallocGEMMContext(c)


def test_grouped_full_mix_matches_plain_path_and_oracle():
    """The 512-problem mix: grouped graph replay == plain per-problem path == the oracle, for every problem."""
    import torch
    mix = datagen.grouped_mix()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1234)
    ops = [(datagen.torch_operand(gen, M, K, wA, eA, "cuda"), datagen.torch_operand(gen, N, K, wB, eB, "cuda"))
           for (M, K, N, wA, eA, wB, eB) in mix]
    plain = make_contexts(mix)
    grouped = make_contexts(mix)
    s = torch.cuda.Stream()
    g = Group(grouped)
    try:
        with torch.cuda.stream(s):
            for c, (a, b) in zip(plain, ops):
                c.lhs.importRegular(a, stream=s)
                c.rhs.importRegular(b, stream=s)
                gemmBitSerial(c, stream=s)
            g.capture([a for a, _ in ops], [b for _, b in ops], stream=s)
            g.replay(stream=s)
        s.synchronize()
        assert g.status(s) == _capi.GBS_OK
        for i, (cp, cg) in enumerate(zip(plain, grouped)):
            assert np.array_equal(cp.res, cg.res), mix[i]
        threads = max(1, min(16, os.cpu_count() or 1))
        for i, (M, K, N, wA, eA, wB, eB) in enumerate(mix):
            A, B = ops[i][0].cpu().numpy(), ops[i][1].cpu().numpy()
            want = O.oracle_gemm(A, B, wA, wB, eA != "u", eB != "u", threads=threads)
            assert np.array_equal(grouped[i].res.reshape(N, M), want), (i, mix[i])
    finally:
        g.free()
        for c in plain + grouped:
            deallocGEMMContext(c)


def test_grouped_rejects_bad_descriptors_without_faulting(lib):
    import torch
    mix = [(40, 640, 300, 2, "u", 3, "s"), (7, 256, 90, 1, "b", 4, "s")]
    ctxs = make_contexts(mix)
    ops = [(torch.ones(M, K, dtype=torch.int8, device="cuda"), torch.ones(N, K, dtype=torch.int8, device="cuda"))
           for (M, K, N, *_r) in mix]
    g = Group(ctxs)
    try:
        g.import_([a for a, _ in ops], [b for _, b in ops])
        assert lib.gbs_debug_group_poison_tile(g._h, 0) == _capi.GBS_OK
        g.gemm()
        torch.cuda.synchronize()
        assert g.status() == _capi.GBS_EINVAL
        assert b"rejected" in lib.gbs_last_error()
        # the context stays usable
        res = torch.zeros(1, device="cuda")
        assert float((res + 1).item()) == 1.0
    finally:
        g.free()
        for c in ctxs:
            deallocGEMMContext(c)


def test_grouped_capture_rejects_the_legacy_stream(lib):
    mix = [(40, 640, 300, 2, "u", 3, "s")]
    ctxs = make_contexts(mix)
    g = Group(ctxs)
    try:
        assert lib.gbs_group_capture(g._h, None, None, None, None) == _capi.GBS_EINVAL
        assert b"legacy default stream" in lib.gbs_last_error()
    finally:
        g.free()
        deallocGEMMContext(ctxs[0])


def test_grouped_rejects_host_sources():
    mix = [(4, 64, 4, 1, "u", 1, "u")]
    ctxs = make_contexts(mix)
    g = Group(ctxs)
    try:
        import ctypes as C
        A = np.ones((4, 64), np.int8)
        L = (C.c_void_p * 1)(A.ctypes.data)
        rc = _capi.load().gbs_group_import(g._h, L, L, None, None)
        assert rc == _capi.GBS_EINVAL
        with pytest.raises(_capi.GBSError):
            g.gemm()  # nothing imported yet
    finally:
        g.free()
        deallocGEMMContext(ctxs[0])


def test_caffenet_chain_as_a_group():
    """The reference's CaffeNet chain (benchmark.cpp:174-237): 8 GEMMs / GEMVs, 2-bit x 2-bit
    unsigned, run as one group (and its graph); every result equals the oracle's."""
    import torch
    mix = datagen.caffenet_mix()
    host = [(datagen.operand(datagen.SEED_BASE + 900 + 2 * i, M, K, wA, eA),
             datagen.operand(datagen.SEED_BASE + 901 + 2 * i, N, K, wB, eB))
            for i, (M, K, N, wA, eA, wB, eB) in enumerate(mix)]
    ctxs = make_contexts(mix)
    dev = [(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()) for A, B in host]
    g = Group(ctxs)
    try:
        st = g.stats()
        assert st["popc_problems"] + st["tc_problems"] == len(mix)
        g.import_([a for a, _ in dev], [b for _, b in dev])
        g.gemm()
        torch.cuda.synchronize()
        assert g.status() == _capi.GBS_OK
        want = [O.oracle_gemm(A, B, 2, 2, False, False, threads=8) for A, B in host]
        for (M, K, N, *_r), c, w in zip(mix, ctxs, want):
            assert np.array_equal(c.res.reshape(N, M), w), (M, K, N)
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            g.capture([a for a, _ in dev], [b for _, b in dev], stream=s)
            g.replay(stream=s)
        s.synchronize()
        for (M, K, N, *_r), c, w in zip(mix, ctxs, want):
            assert np.array_equal(c.res.reshape(N, M), w), (M, K, N)
    finally:
        g.free()
        for c in ctxs:
            deallocGEMMContext(c)
