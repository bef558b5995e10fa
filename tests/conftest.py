import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session", autouse=True)
def _built_library():
    """Build libxtg.so and the oracle once (incremental) before any test."""
    from xtensor_gb300.build import build
    build()
    yield
