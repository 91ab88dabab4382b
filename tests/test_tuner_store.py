"""Autotuner store: versioned text file, save/load round trip, entries from
another version ignored.  No GPU needed."""


def test_store_roundtrip_and_version_check(gbs_lib, tmp_path):
    from gemmbitserial_gb300 import _capi
    lib = gbs_lib
    assert lib.gbs_tuner_clear() == _capi.GBS_OK
    path = str(tmp_path / "tuner.txt").encode()
    # a store with two entries written by hand in the current format
    (tmp_path / "tuner.txt").write_text("gbs-tuner v1 sm_103a\n"
                                        "5 5 6 3 2 0 1 3 256 151.5\n"
                                        "0 3 6 1 1 0 0 1 -1 2.0\n"
                                        "garbage line\n")
    assert lib.gbs_tuner_load(path, 1) == _capi.GBS_OK
    assert lib.gbs_tuner_entries() == 2
    out = str(tmp_path / "again.txt").encode()
    assert lib.gbs_tuner_save(out) == _capi.GBS_OK
    lines = (tmp_path / "again.txt").read_text().splitlines()
    assert lines[0] == "gbs-tuner v1 sm_103a" and len(lines) == 3
    # another version: rejected, nothing replaced
    (tmp_path / "old.txt").write_text("gbs-tuner v0 sm_100a\n1 1 1 1 1 0 0 1 -1 1.0\n")
    assert lib.gbs_tuner_load(str(tmp_path / "old.txt").encode(), 1) == _capi.GBS_EINVAL
    assert b"another version" in lib.gbs_last_error()
    assert lib.gbs_tuner_entries() == 2
    assert lib.gbs_tuner_load(str(tmp_path / "missing.txt").encode(), 0) == _capi.GBS_EINVAL
    assert lib.gbs_tuner_clear() == _capi.GBS_OK and lib.gbs_tuner_entries() == 0


def test_committed_gb300_store_parses():
    """The committed store is in the current format: a version line, then entries of 7 key integers,
    a pipe, a variant and a time, one for every named workload's shape class."""
    import os

    from gemmbitserial_gb300 import datagen
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lines = open(os.path.join(root, "gemmbitserial_gb300", "tuned", "gb300_sm103a.txt")).read().splitlines()
    assert lines[0] == "gbs-tuner v1 sm_103a"
    entries = [l.split() for l in lines[1:] if l.strip()]
    assert len(entries) == len(datagen.WORKLOADS)  # the named workloads have distinct shape classes
    for e in entries:
        assert len(e) == 10 and 1 <= int(e[7]) <= 5 and float(e[9]) > 0
