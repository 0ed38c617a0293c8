import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 library)")


def pytest_collection_modifyitems(config, items):
    # keep the CPU suite usable on machines without a GPU
    pass


@pytest.fixture(scope="session")
def oracle_lib():
    import pyoracle

    pyoracle.load()
    return pyoracle
