import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built engine")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))


def import_stock_reference():
    from bench import import_stock_reference as load
    return load()


@pytest.fixture(scope="session")
def stock_reference():
    ref = import_stock_reference()
    if ref is None:
        pytest.skip("the stock reference is not installed under baseline/_ref")
    return ref
