import importlib
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

PKG_NAME = "modgcd-onegpu_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _built():
    """Builds the library and the oracle once per session (cheap when up to date)."""
    pkg = importlib.import_module(PKG_NAME)
    pkg.build()
    import pyoracle
    pyoracle.build()
    return pkg


@pytest.fixture(scope="session")
def mgcd():
    return _built()


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


B62 = "0123456789ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz"


def parse_b62(s):
    x = 0
    for ch in s.strip():
        x = x * 62 + B62.index(ch)
    return x


def golden_pairs(case):
    """(u, v) pairs of a golden file in the reference's base-62 test-vector format."""
    lines = [ln for ln in open(os.path.join(GOLDEN, case["file"])).read().split("\n") if ln.strip()]
    return [(parse_b62(lines[2 * i]), parse_b62(lines[2 * i + 1])) for i in range(len(lines) // 2)]


@pytest.fixture(scope="session")
def device(mgcd):
    dev = mgcd.Device(0, 32)
    yield dev
    dev.close()
