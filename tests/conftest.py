import json
import lzma
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.join(ROOT, "tests")
GOLDEN = os.path.join(TESTS, "golden")
PKG = os.path.join(ROOT, "volume-compressor_gb300")
for p in (TESTS, GOLDEN, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103a) device")
    config.addinivalue_line("markers", "slow: long-running (full-size workload)")


def _ensure_built():
    import vc_gb300
    vc_gb300.build()
    import oraclelib
    oraclelib.build()


@pytest.fixture(scope="session")
def vc():
    _ensure_built()
    import vc_gb300
    return vc_gb300


@pytest.fixture(scope="session")
def oracle():
    _ensure_built()
    import oraclelib
    return oraclelib


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        cases = json.load(f)["cases"]
    return {c["name"]: c for c in cases}


def load_archive(case):
    with open(os.path.join(GOLDEN, case["file"]), "rb") as f:
        return lzma.decompress(f.read())


@pytest.fixture(scope="session")
def gpu(vc):
    s, nsm, cc = vc.device_info()
    if s != 0:
        pytest.fail(f"no usable CUDA device: {vc.last_error()}")
    return {"num_sms": nsm, "cc": cc}
