import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path)")


@pytest.fixture(scope="session")
def bmg():
    """The product package with its CUDA library built in-tree."""
    import bmagwa_gb300 as bg
    bg.build()
    return bg


@pytest.fixture(scope="session")
def oracle():
    import oracle.port as op
    op.lib()
    return op
