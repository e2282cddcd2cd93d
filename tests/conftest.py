import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libsvgpu.so")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def golden_ordering():
    return load_golden("ordering")


@pytest.fixture(scope="session")
def golden_likelihood():
    return load_golden("likelihood")


@pytest.fixture(scope="session")
def golden_blocks():
    return load_golden("blocks")


@pytest.fixture(scope="session")
def golden_gp():
    return load_golden("gp")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o
