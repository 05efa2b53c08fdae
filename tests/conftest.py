import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103) and the built library")


@pytest.fixture(scope="session")
def gpulib():
    """The GPU library; fails loudly (no fallback) when it is not built."""
    import nfft_gb300
    return nfft_gb300.lib()


@pytest.fixture(scope="session")
def refrun():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "refrun.npz")))


@pytest.fixture(scope="session")
def testdata():
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, "reference_testdata.npz")))
