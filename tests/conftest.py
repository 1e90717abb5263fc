import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
DATA = os.path.join(GOLDEN, "data")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity of the CUDA library against the oracle)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """the oracle and the generator are host code: build them for every run"""
    from bruno_gb300 import build
    from oracle import oracle
    oracle.build()
    build.build_synth()
    yield


def fixture_bytes(name: str) -> bytes:
    with open(os.path.join(DATA, name), "rb") as f:
        return f.read()
