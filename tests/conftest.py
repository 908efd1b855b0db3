import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "last: runs after every other test (GPU paths not yet run on a GB300, "
                                       "so that a failure under -x does not stop the established suites)")


def pytest_collection_modifyitems(config, items):
    items.sort(key=lambda it: it.get_closest_marker("last") is not None)   # stable: order kept within groups


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "qg1l_golden.npz")))
