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


REF_INSTALL = os.path.join(ROOT, "baseline", "_ref")


def import_stock_reference():
    """The reference package as installed under baseline/_ref (pip --target),
    or None.  Its plotting and pandas imports are served by empty stand-in
    modules for the import only; the reference keeps its own bindings."""
    import importlib
    import types
    if not os.path.isdir(os.path.join(REF_INSTALL, "pyatmosphere")):
        return None
    added = []
    for name in ("matplotlib", "matplotlib.pyplot", "pandas"):
        if name not in sys.modules:
            sys.modules[name] = types.ModuleType(name)
            added.append(name)
    if "matplotlib.pyplot" in added:
        sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    if REF_INSTALL not in sys.path:
        sys.path.append(REF_INSTALL)
    try:
        ref = importlib.import_module("pyatmosphere")
        for sub in ("channels", "grids", "sources", "pathes", "phase_screens", "pupils", "measures",
                    "theory.models", "simulations", "simulations.simulation", "simulations.pdt",
                    "simulations.beam", "utils"):
            importlib.import_module("pyatmosphere." + sub)
    finally:
        for name in added:
            sys.modules.pop(name, None)
    ref.gpu.config["use_gpu"] = False
    return ref


@pytest.fixture(scope="session")
def stock_reference():
    ref = import_stock_reference()
    if ref is None:
        pytest.skip("the stock reference is not installed under baseline/_ref")
    return ref
