import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libespic")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="session")
def po():
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle


def _espic_module():
    import importlib
    return importlib.import_module("plasma-simulations-by-example_gb300")


@pytest.fixture(scope="session")
def espic():
    """The ctypes view of libespic on a GPU (built on first use)."""
    mod = _espic_module()
    import os as _os
    if not _os.path.exists(mod.LIB_PATH):
        mod.build()
    mod.lib()
    return mod
