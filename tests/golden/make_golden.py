"""Regenerates the golden fixtures in this directory from the reference.

Run where the reference sources exist (it reads them; the fixtures it writes
travel with the repository):

    python tests/golden/make_golden.py REFDIR   # compiles the unmodified reference from REFDIR first

Writes
  mnist_kat.npz   -- the reference's known-answer test (test/mnistdata.h,
                     used by test/test.cpp:157-172): bipolar weights packed one
                     bit per value, the 2-bit input vector, the golden result.
  ref_vectors.json, ref_results_small.npz -- seeds, input hashes and the
                     reference's results (in full when small, else sha256) for the
                     reference's own test grids (test/test.cpp:30-277) plus
                     cases it never covers (signed x signed, unsigned x signed,
                     col-major import, wide element types, masked
                     out-of-range values, odd shapes, K not a multiple of 64).
  ref_configs.json-- sha256 of the reference's int32 results on the full-size
                     benchmark workloads (seeded by gemmbitserial_gb300.datagen).
  ref_float_import.npz -- importRegular<float> through the reference, then
                     exportRegular, for every width and encoding.
  ref_quantize.npz -- importRegularAndQuantize (gemmbitserial.hpp:282-305) through
                     the reference, then exportRegular: inputs, thresholds
                     [nThres][rows] and the resulting values, for every element
                     type, sorted and unsorted thresholds, no thresholds, more
                     levels than the bit width holds, and column-major input.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gemmbitserial_gb300 import datagen  # noqa: E402
from oracle import oracle as O  # noqa: E402


def parse_array(text: str, name: str) -> np.ndarray:
    m = re.search(name + r"\[\]\s*=\s*\{(.*?)\};", text, re.S)
    return np.array([int(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()], np.int64)


def make_mnist(refdir: str) -> None:
    text = open(os.path.join(refdir, "test", "mnistdata.h")).read()
    defs = dict(re.findall(r"#define\s+(MNIST_\w+)\s+(\w+)", text))
    n_in, n_out = int(defs["MNIST_IN"]), int(defs["MNIST_OUT"])
    x = parse_array(text, "mnist_in").astype(np.uint8)
    w = parse_array(text, "mnist_weights")
    golden = parse_array(text, "mnist_res_golden").astype(np.int32)
    assert x.size == n_in and w.size == n_in * n_out and golden.size == n_out
    assert set(np.unique(w)) <= {-1, 1}, "weights are expected to be bipolar"
    np.savez_compressed(os.path.join(HERE, "mnist_kat.npz"),
                        w_bits=np.packbits((w > 0).astype(np.uint8)), x=x, golden=golden,
                        shape=np.array([n_out, n_in], np.int64),
                        flags=np.array([int(defs["MNIST_WBITS"]), int(defs["MNIST_ABITS"]),
                                        int(defs["MNIST_WSIGN"] == "true"), int(defs["MNIST_ASIGN"] == "true")]))


def cases():
    """(name, M, K, N, wA, sA, wB, sB, dtA, dtB, cmA, cmB, value-range-kind)."""
    dims = [3, 5, 7, 16, 17, 18, 30, 31, 32, 100, 177]
    # test_matrix_matrix (test.cpp:110-155): unsigned uint8, d x 2d x 3d and d x 2d x 1
    for b in (2, 3, 4):
        for d in dims:
            for mv in (0, 1):
                yield (f"mm_b{b}_d{d}_mv{mv}", d, 2 * d, 1 if mv else 3 * d, b, 0, b, 0, "u8", "u8", 0, 0, "in")
    # test_bipolar_times_regular (test.cpp:174-235): d x d x d, swapped and not
    for sw in (0, 1):
        for b in (2, 3, 4):
            for d in dims:
                for sg in (1, 0):
                    if sw:
                        yield (f"bpreg_sw_b{b}_d{d}_s{sg}", d, d, d, b, sg, 1, 1, "i8", "i8", 0, 0, "in")
                    else:
                        yield (f"bpreg_b{b}_d{d}_s{sg}", d, d, d, 1, 1, b, sg, "i8", "i8", 0, 0, "in")
    # test_bipolar_times_bipolar (test.cpp:237-277)
    for d in dims:
        for mv in (0, 1):
            yield (f"bpbp_d{d}_mv{mv}", d, d, 1 if mv else d, 1, 1, 1, 1, "i8", "i8", 0, 0, "in")
    # beyond the reference's tests
    rng = np.random.default_rng(7)
    for t in range(96):
        M, K, N = int(rng.integers(1, 90)), int(rng.integers(1, 700)), int(rng.integers(1, 90))
        if t % 8 == 0:
            N = 1
        wA, wB = int(rng.integers(1, 9)), int(rng.integers(1, 9))
        sA, sB = int(rng.integers(0, 2)), int(rng.integers(0, 2))
        dtA = ["i8", "u8", "i16", "i32"][t % 4]
        dtB = ["i8", "u8", "i16", "i32"][(t // 4) % 4]
        yield (f"mix{t}", M, K, N, wA, sA, wB, sB, dtA, dtB, t % 3 == 0, t % 5 == 0, "wide" if t % 2 else "in")


NP = {"i8": np.int8, "u8": np.uint8, "i16": np.int16, "i32": np.int32}


def operand(seed, rows, cols, bits, sgn, dt, kind):
    if kind == "wide":  # values outside the encodable range: the import masks them
        lo, hi = {"i8": (-128, 127), "u8": (0, 255), "i16": (-700, 700), "i32": (-100000, 100000)}[dt]
        return datagen.uniform_int(seed, (rows, cols), lo, hi, np.int64).astype(NP[dt])
    if bits == 1 and sgn:
        return datagen.bipolar(seed, (rows, cols), NP[dt]) if dt != "u8" else datagen.uniform_int(seed, (rows, cols), 0, 1, np.uint8)
    enc = "s" if sgn else "u"
    v = datagen.operand(seed, rows, cols, bits, enc, np.int64)
    return v.astype(NP[dt])


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


SMALL = 2048  # results up to this many elements are stored in full, larger ones as sha256


def make_vectors() -> None:
    full = {}
    meta = []
    for idx, (name, M, K, N, wA, sA, wB, sB, dtA, dtB, cmA, cmB, kind) in enumerate(cases()):
        seed = datagen.SEED_BASE + 0x10000 + idx * 2
        A = operand(seed, M, K, wA, sA, dtA, kind)
        B = operand(seed + 1, N, K, wB, sB, dtB, kind)
        Ain = np.ascontiguousarray(A.T) if cmA else A
        Bin = np.ascontiguousarray(B.T) if cmB else B
        res, dims, _ = O.ref_gemm(Ain, Bin, wA, wB, sA, sB, bool(cmA), bool(cmB))
        if res.size <= SMALL:
            full[name] = res
        meta.append({"name": name, "M": M, "K": K, "N": N, "wA": wA, "sA": sA, "wB": wB, "sB": sB,
                     "dtA": dtA, "dtB": dtB, "cmA": int(cmA), "cmB": int(cmB), "kind": kind, "seed": seed,
                     "sha_A": sha(A), "sha_B": sha(B), "sha_res": sha(res), "ref_dims": dims})
    rows = []
    # sumRows and import/export round trips (test.cpp:30-108)
    for b in (1, 2, 3, 4, 7):
        for d in (4, 16, 17, 32, 77, 100, 1023):
            for sg in (1, 0):
                seed = datagen.SEED_BASE + 0x20000 + b * 4096 + d * 2 + sg
                X = operand(seed, d, d, b, sg, "i8", "in")
                rs = np.zeros(d, np.int32)
                rt = np.zeros(d * d, np.int32)
                O.ref().ref_sum_rows(d, d, b, sg, O._ptr(X), O.DT_I8, O._ptr(rs))
                O.ref().ref_roundtrip(d, d, b, sg, O._ptr(X), O.DT_I8, O._ptr(rt))
                rows.append({"b": b, "d": d, "s": sg, "seed": seed, "sha_X": sha(X),
                             "sum": [int(v) for v in rs], "sha_export": sha(rt.reshape(d, d))})
    np.savez_compressed(os.path.join(HERE, "ref_results_small.npz"), **full)
    with open(os.path.join(HERE, "ref_vectors.json"), "w") as f:
        json.dump({"gemm": meta, "rows": rows}, f, separators=(",", ":"))


QUANTIZE_CASES = [  # rows, cols, bits, nThres, sorted thresholds, column-major
    (5, 70, 2, 3, True, False), (17, 130, 3, 7, True, True), (8, 64, 2, 7, True, False),
    (9, 33, 4, 0, True, False), (4, 100, 1, 1, False, False), (6, 77, 3, 5, False, True),
    (1, 1, 2, 2, True, False), (33, 65, 8, 20, True, False), (64, 300, 4, 15, True, False),
    (40, 257, 2, 3, True, True),
]


def make_quantize() -> None:
    out = {}
    dts = [np.int8, np.uint8, np.int16, np.int32, np.float32]
    for i, (rows, cols, bits, nthres, srt, cm) in enumerate(QUANTIZE_CASES):
        for dt in dts:
            rng = np.random.default_rng(1000 * i + dts.index(dt))
            if dt == np.float32:
                a = rng.normal(0, 3, (rows, cols)).astype(dt)
                if nthres == 0:  # (uint8_t)float is only defined for values in [0, 256)
                    a = rng.integers(0, 256, (rows, cols)).astype(dt)
                t = rng.normal(0, 3, (nthres, rows)).astype(dt)
            else:
                info = np.iinfo(dt)
                lo, hi = max(int(info.min), -1000), min(int(info.max), 1000)
                a = rng.integers(lo, hi + 1, (rows, cols)).astype(dt)
                t = rng.integers(lo, hi + 1, (nthres, rows)).astype(dt)
            if srt:
                t = np.sort(t, axis=0)
            src = np.ascontiguousarray(a.T) if cm else a
            key = f"q{i}_{np.dtype(dt).name}"
            out[key + "_src"] = src
            out[key + "_thr"] = t
            out[key + "_meta"] = np.array([rows, cols, bits, nthres, int(cm)], np.int64)
            out[key + "_values"] = O.ref_quantize_values(src, t, bits, cm)
    np.savez_compressed(os.path.join(HERE, "ref_quantize.npz"), **out)


def make_float_import() -> None:
    """importRegular<float> (quantize<float>, gemmbitserial.hpp:170-186) through the reference,
    then exportRegular: values inside each encoding's defined range, fractions included."""
    out = {}
    i = 0
    for bits in (1, 2, 3, 4, 8):
        for sgn in (False, True):
            for rows, cols in ((7, 70), (33, 129), (1, 5)):
                rng = np.random.default_rng(5000 + i)
                if sgn and bits > 1:
                    lo, hi = -(1 << (bits - 1)), 1 << (bits - 1)
                elif sgn:
                    lo, hi = -3, 3
                else:
                    lo, hi = 0, min(256, 1 << bits)
                a = rng.uniform(lo, hi - 1e-3, (rows, cols)).astype(np.float32)
                a[0, :min(3, cols)] = [lo, 0.0, -0.0][:min(3, cols)]
                key = f"f{i}"
                out[key + "_src"] = a
                out[key + "_meta"] = np.array([bits, int(sgn)], np.int64)
                out[key + "_values"] = O.ref_import_values(a, bits, sgn)
                i += 1
    np.savez_compressed(os.path.join(HERE, "ref_float_import.npz"), **out)


def make_config_hashes() -> None:
    res = {}
    for name in datagen.WORKLOADS:
        M, K, N, wA, sA, wB, sB, A, B = datagen.workload(name)
        r, dims, _ = O.ref_gemm(A, B, wA, wB, sA, sB)
        res[name] = {"sha256": hashlib.sha256(np.ascontiguousarray(r).tobytes()).hexdigest(),
                     "first": [int(x) for x in r.ravel()[:8]], "sum": int(r.astype(np.int64).sum()),
                     "dims": dims}
    with open(os.path.join(HERE, "ref_configs.json"), "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    refdir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFDIR")
    if not refdir or not os.path.isfile(os.path.join(refdir, "gemmbitserial.hpp")):
        sys.exit("usage: make_golden.py REFDIR   (or REFDIR=... in the environment): the reference checkout")
    os.environ["REFDIR"] = refdir  # the oracle Makefile builds the reference from there
    if not O.ref_available():
        O.build(ref=True)
    make_mnist(refdir)
    make_vectors()
    make_quantize()
    make_float_import()
    make_config_hashes()
    print("golden fixtures written to", HERE)
