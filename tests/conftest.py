import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as _oracle  # noqa: F401  (oracle/oracle.py)
    _oracle.lib()
    return _oracle


@pytest.fixture(scope="session")
def felib():
    from cm_gb300 import _lib
    return _lib.load()
