import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 (GB300) CUDA device")


def _has_gpu():
    try:
        import largetb_gb300 as T
        c = T.Context()
        c.close()
        return True
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not _has_gpu():
        pytest.fail("no usable sm_103 device or libtb_gb300.so failed to load")
    import largetb_gb300 as T
    return T


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "reference_dumps.npz"))


def dense_coo(g, key):
    import numpy as np
    A = np.zeros(tuple(g[key + "_shape"]))
    A[g[key + "_r"], g[key + "_c"]] = g[key + "_v"]
    return A
