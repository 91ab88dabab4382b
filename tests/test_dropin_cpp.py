"""The C++ drop-in header: code written against the reference's API compiles
against include/gemmbitserial.hpp, links libgbs.so and gives the reference's
results (groups of test/test.cpp, compared in full)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_dropin(tmpdir):
    exe = os.path.join(tmpdir, "dropin_test")
    lib_dir = os.path.join(ROOT, "gemmbitserial_gb300")
    subprocess.run(["g++", "-O2", "-std=c++11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "dropin", "dropin_test.cpp"), "-o", exe,
                    "-L", lib_dir, "-lgbs", f"-Wl,-rpath,{lib_dir}"], check=True)
    return exe


def test_dropin_header_compiles_and_links(gbs_lib, tmp_path):
    assert os.path.exists(build_dropin(str(tmp_path)))


@pytest.mark.gpu
def test_dropin_reference_test_groups(gbs_lib, tmp_path):
    exe = build_dropin(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "All tests completed successfully" in r.stdout
