"""The C-ABI library loads and exports every entry point include/gbs.h declares.
No compute calls here: these run without a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"GBS_API[^;(]*?\b(gbs_\w+)\s*\(", text)))


def test_header_declares_the_hot_path():
    names = declared("gbs.h")
    for n in ["gbs_ctx_alloc", "gbs_import", "gbs_gemm", "gbs_get_result", "gbs_ctx_free"]:
        assert n in names


def test_every_declared_symbol_is_exported(gbs_lib):
    lib = C.CDLL(os.path.join(ROOT, "gemmbitserial_gb300", "libgbs.so"))
    for header in sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")):
        for name in declared(header):
            assert hasattr(lib, name), f"{name} declared in {header} but not exported"


def test_ctypes_binding_covers_header(gbs_lib):
    from gemmbitserial_gb300 import _capi
    assert set(declared("gbs.h")) <= set(_capi.SIGNATURES)


def test_version_string(gbs_lib):
    assert b"sm_103a" in gbs_lib.gbs_version()


def test_bad_widths_rejected_before_any_device_work(gbs_lib):
    from gemmbitserial_gb300 import _capi
    h = C.c_void_p()
    for wa, wb in [(0, 1), (9, 1), (1, 0), (3, 12)]:
        rc = gbs_lib.gbs_ctx_alloc(4, 64, 4, wa, wb, 0, 0, C.byref(h))
        assert rc == _capi.GBS_EINVAL
        assert b"bit widths" in gbs_lib.gbs_last_error()
    assert gbs_lib.gbs_ctx_alloc(4, 64, 4, 1, 1, 0, 0, None) == _capi.GBS_EINVAL


def test_null_context_is_rejected(gbs_lib):
    from gemmbitserial_gb300 import _capi
    assert gbs_lib.gbs_gemm(None, None) == _capi.GBS_EINVAL
    assert gbs_lib.gbs_import(None, 0, None, 0, 0, None) == _capi.GBS_EINVAL
    assert gbs_lib.gbs_ctx_free(None) == _capi.GBS_OK
    for mode in (_capi.GBS_HOST_IMPORT_AUTO, _capi.GBS_HOST_IMPORT_STAGED):
        assert gbs_lib.gbs_set_host_import(None, mode) == _capi.GBS_EINVAL
    assert b"gbs_set_host_import" in gbs_lib.gbs_last_error()
    assert gbs_lib.gbs_set_variant(None, 4) == _capi.GBS_EINVAL
    assert gbs_lib.gbs_debug_group_tc_kernel(None) < 0


def test_python_api_fails_loudly_without_library(monkeypatch, tmp_path):
    from gemmbitserial_gb300 import _capi
    monkeypatch.setattr(_capi, "_lib", None)
    monkeypatch.setattr(_capi, "lib_path", lambda: str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError, match="not built"):
        _capi.load()


def test_context_padding_is_the_references(gbs_lib):
    """gbs_ctx_dims (host arithmetic, no device) gives the reference's lhs/rhs nrows_a, ncols_a and
    cache blocks for every golden vector and full-size workload, as the compiled reference recorded."""
    import json

    from gemmbitserial_gb300 import datagen
    gold = os.path.join(ROOT, "tests", "golden")
    cases = [((v["M"], v["K"], v["N"]), v["ref_dims"]) for v in json.load(open(os.path.join(gold, "ref_vectors.json")))["gemm"]]
    cfg = json.load(open(os.path.join(gold, "ref_configs.json")))
    cases += [((M, K, N), cfg[name]["dims"]) for name, (M, K, N, _a, _b) in datagen.WORKLOADS.items()]
    for (M, K, N), want in cases:
        out = (C.c_uint64 * 6)()
        assert gbs_lib.gbs_ctx_dims(M, K, N, out) == 0
        assert list(out) == want, (M, K, N)
    # degenerate sides pad to nothing; matrix-vector depth pads to 256 bits
    out = (C.c_uint64 * 6)()
    assert gbs_lib.gbs_ctx_dims(0, 100, 5, out) == 0 and out[0] == 0 and out[2] == 128
    assert gbs_lib.gbs_ctx_dims(10, 100, 1, out) == 0 and out[2] == 256
