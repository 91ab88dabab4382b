"""The oracle (C restatement of the reference) pinned against the reference's
own known-answer test and golden vectors produced by the unmodified
reference (tests/golden/make_golden.py)."""
import hashlib
import json
import os

import numpy as np
import pytest

import make_golden as G
from gemmbitserial_gb300 import datagen
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load_mnist():
    z = np.load(os.path.join(GOLD, "mnist_kat.npz"))
    n_out, n_in = [int(v) for v in z["shape"]]
    w = np.unpackbits(z["w_bits"])[: n_out * n_in].reshape(n_out, n_in).astype(np.int8) * 2 - 1
    return w, z["x"], z["golden"], [int(v) for v in z["flags"]]


def test_mnist_known_answer():
    """test/test.cpp:157-172: 256x784 bipolar weights x 2-bit input vector (GEMV, bipolar x regular)."""
    w, x, golden, (wb, ab, ws, as_) = load_mnist()
    res = O.oracle_gemm(w, x.reshape(1, -1), wb, ab, ws, as_)
    assert np.array_equal(res.ravel(), golden)


def test_datagen_is_pinned():
    """The seeded generator the fixtures depend on must not drift."""
    r = datagen.splitmix64(0, 3)
    assert [int(v) for v in r] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


VEC = json.load(open(os.path.join(GOLD, "ref_vectors.json")))
SMALL = np.load(os.path.join(GOLD, "ref_results_small.npz"))


def regen(c):
    A = G.operand(c["seed"], c["M"], c["K"], c["wA"], c["sA"], c["dtA"], c["kind"])
    B = G.operand(c["seed"] + 1, c["N"], c["K"], c["wB"], c["sB"], c["dtB"], c["kind"])
    assert sha(A) == c["sha_A"] and sha(B) == c["sha_B"], "input generator drifted"
    Ain = np.ascontiguousarray(A.T) if c["cmA"] else A
    Bin = np.ascontiguousarray(B.T) if c["cmB"] else B
    return A, B, Ain, Bin


@pytest.mark.parametrize("c", VEC["gemm"], ids=[c["name"] for c in VEC["gemm"]])
def test_oracle_matches_reference_vectors(c):
    A, B, Ain, Bin = regen(c)
    ctx = O.OracleContext(c["M"], c["K"], c["N"], c["wA"], c["wB"], c["sA"], c["sB"])
    ctx.import_(0, Ain, bool(c["cmA"]))
    ctx.import_(1, Bin, bool(c["cmB"]))
    ctx.gemm()
    res = ctx.res()
    assert ctx.dims == c["ref_dims"]
    assert sha(res) == c["sha_res"]
    if c["name"] in SMALL.files:
        assert np.array_equal(res, SMALL[c["name"]])
    # the naive definition (test/testhelpers.hpp:34-45) on the decoded values agrees too
    va = O.decode_values(A, c["wA"], c["sA"], A.dtype == np.uint8)
    vb = O.decode_values(B, c["wB"], c["sB"], B.dtype == np.uint8)
    assert np.array_equal(O.naive_gemm(va, vb), res)


@pytest.mark.parametrize("r", VEC["rows"], ids=[f"b{r['b']}_d{r['d']}_s{r['s']}" for r in VEC["rows"]])
def test_oracle_rowsums_and_export(r):
    """test/test.cpp:30-108 (sumRows, importRegular -> exportRegular), compared in full."""
    X = G.operand(r["seed"], r["d"], r["d"], r["b"], r["s"], "i8", "in")
    assert sha(X) == r["sha_X"]
    ctx = O.OracleContext(r["d"], r["d"], 1, r["b"], 1, r["s"], 0)
    ctx.import_(0, X)
    assert [int(v) for v in ctx.sum_rows(0)] == r["sum"]
    assert sha(ctx.export(0)) == r["sha_export"]


CFG = json.load(open(os.path.join(GOLD, "ref_configs.json")))


@pytest.mark.parametrize("name", sorted(CFG))
def test_oracle_full_size_workloads(name):
    """Full-size benchmark workloads: oracle result hash equals the reference's."""
    M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
    res = O.oracle_gemm(A, B, wA, wB, sA, sB, threads=os.cpu_count() or 4)
    assert sha(res) == CFG[name]["sha256"]


def test_oracle_threaded_equals_serial():
    rng = np.random.default_rng(3)
    for t in range(20):
        M, K, N = [int(v) for v in rng.integers(1, 200, 3)]
        wA, wB = [int(v) for v in rng.integers(1, 5, 2)]
        sA, sB = [int(v) for v in rng.integers(0, 2, 2)]
        A = rng.integers(-8, 8, (M, K)).astype(np.int8)
        B = rng.integers(-8, 8, (N, K)).astype(np.int8)
        assert np.array_equal(O.oracle_gemm(A, B, wA, wB, sA, sB),
                              O.oracle_gemm(A, B, wA, wB, sA, sB, threads=5))


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not compiled here")
def test_oracle_matches_compiled_reference_random():
    rng = np.random.default_rng(11)
    for t in range(150):
        M, N = [int(v) for v in rng.integers(1, 60, 2)]
        K = int(rng.integers(1, 500))
        if t % 6 == 0:
            N = 1
        wA, wB = [int(v) for v in rng.integers(1, 9, 2)]
        sA, sB = [int(v) for v in rng.integers(0, 2, 2)]
        A = rng.integers(-128, 128, (M, K)).astype(np.int8)
        B = rng.integers(0, 256, (N, K)).astype(np.uint8)
        r_ref, dims, planes = O.ref_gemm(A, B, wA, wB, sA, sB, want_planes=True)
        ctx = O.OracleContext(M, K, N, wA, wB, sA, sB)
        ctx.import_(0, A)
        ctx.import_(1, B)
        ctx.gemm()
        pl = np.concatenate([ctx.planes(0).ravel(), ctx.planes(1).ravel()])
        assert np.array_equal(ctx.res(), r_ref) and ctx.dims == dims
        assert np.array_equal(pl, planes[: pl.size])


def quantize_cases():
    z = np.load(os.path.join(GOLD, "ref_quantize.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    return [(k, z[k + "_src"], z[k + "_thr"], z[k + "_meta"], z[k + "_values"]) for k in keys]


def test_quantize_oracle_matches_reference_fixtures():
    """importRegularAndQuantize (gemmbitserial.hpp:282-305): the C restatement against the
    reference's own results for every element type, unsorted and empty threshold sets,
    more levels than the width holds, and column-major input."""
    cases = quantize_cases()
    assert len(cases) >= 50
    for key, src, thr, meta, want in cases:
        rows, cols, bits, nthres, cm = (int(x) for x in meta)
        assert thr.shape == (nthres, rows)
        got = O.quantize_values(src, thr, bits, bool(cm))
        assert np.array_equal(got, want), key
        if O.ref_available():
            assert np.array_equal(O.ref_quantize_values(src, thr, bits, bool(cm)), want), key


def test_quantize_oracle_rejects_signed():
    ctx = O.OracleContext(4, 64, 4, 2, 2, True, False)
    with pytest.raises(ValueError):
        ctx.import_quantize(0, np.zeros((4, 64), np.int8), np.zeros((1, 4), np.int8))


def test_float_import_oracle_matches_reference_fixtures():
    """importRegular<float> (quantize<float>, gemmbitserial.hpp:170-186): the C restatement
    against the reference's own results, fractional and negative values included."""
    z = np.load(os.path.join(GOLD, "ref_float_import.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    assert len(keys) >= 30
    for k in keys:
        bits, sgn = (int(x) for x in z[k + "_meta"])
        got = O.import_values(z[k + "_src"], bits, bool(sgn))
        assert np.array_equal(got, z[k + "_values"]), k
        if O.ref_available():
            assert np.array_equal(O.ref_import_values(z[k + "_src"], bits, bool(sgn)), z[k + "_values"]), k
