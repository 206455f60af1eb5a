import ctypes
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402

ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libavbd_ref.so")
GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_runs.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def pkg():
    return entry.load_package()


@pytest.fixture(scope="session")
def oracle(pkg):
    """The CPU restatement of the reference step (the parity checker)."""
    if not os.path.exists(ORACLE_LIB):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return pkg.capi.Api(ctypes.CDLL(ORACLE_LIB), "avbdo_")


@pytest.fixture(scope="session")
def ref(pkg):
    """The reference solver compiled from its own sources (only where those sources exist)."""
    if not os.path.exists(REF_LIB):
        pytest.skip("compiled reference not present on this machine")
    return pkg.capi.Api(ctypes.CDLL(REF_LIB), "avbdr_")


@pytest.fixture(scope="session")
def gpu(pkg):
    """The GPU library. Fails (never skips) when it is missing: there is no fallback path."""
    return pkg.gpu_api()


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)
