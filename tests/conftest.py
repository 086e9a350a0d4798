"""Test configuration.  ``gpu`` marks tests that need a CUDA device; the
reference's own fixtures (``tests/conftest.py:13-85`` of GIGA-Lens) are
restated in ``tests/helpers.py``."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture
def default_prior():
    from tests.helpers import default_prior as f
    return f()


@pytest.fixture
def default_physmodel():
    from tests.helpers import default_physmodel as f
    return f()


@pytest.fixture
def default_data():
    import numpy as np
    return np.zeros((20, 20)), 0.1, 100
