import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
PKG_NAME = "engineering-degree-in-plasma-simulations_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA library")


@pytest.fixture(scope="session")
def pic():
    """The package (hyphenated directory name, imported through importlib)."""
    return importlib.import_module(PKG_NAME)


@pytest.fixture(scope="session")
def port():
    import oracle

    oracle.build_port()
    return oracle.Port()


def golden(name):
    import numpy as np

    return dict(np.load(os.path.join(ROOT, "tests", "golden", name + ".npz")))
