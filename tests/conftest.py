import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "sci-solver_peridynamic_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def pdgb():
    """The package (hyphenated directory name, imported by path)."""
    return importlib.import_module(PKG_NAME)


@pytest.fixture(scope="session")
def scenes():
    return importlib.import_module(PKG_NAME + ".scenes")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build_oracle()
    return O
