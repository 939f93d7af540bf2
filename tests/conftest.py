import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built extension")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "reference_fixtures.npz")))


@pytest.fixture(scope="session")
def extended():
    """Extended-precision (80-bit) runs of periodic cases, made by
    tests/golden/make_extended.py."""
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "extended_precision.npz")))
