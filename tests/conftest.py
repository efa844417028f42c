"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device (GB300); the rest
run on CPU: the oracle against the golden vectors, the host logic, and the
C-ABI library's load and exports."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def built_lib():
    from v119_2025_12_19_hexatop_aws_gb300 import build as b
    return b.build()


@pytest.fixture(scope="session")
def ctx(built_lib):
    from v119_2025_12_19_hexatop_aws_gb300 import _lib
    c = _lib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def oracle():
    from oracle import reference
    reference.lib()
    return reference


@pytest.fixture
def rng():
    return np.random.default_rng(1234)
