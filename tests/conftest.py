import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on a GB300)")


@pytest.fixture(scope="session", autouse=True)
def built_oracle():
    """The oracle's C restatement is compiled once per session (it is the checker)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)


@pytest.fixture(scope="session")
def gbs_lib():
    """libgbs.so, built in tree if missing."""
    from gemmbitserial_gb300 import _capi, build
    build.build()
    return _capi.load()
