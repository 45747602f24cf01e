import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "reference_unittests.npz"))


@pytest.fixture(scope="session")
def tgv_reference():
    import numpy as np
    d = np.load(os.path.join(ROOT, "tests", "golden", "tgv_split_reference.npz"))
    return d["header"], d["rows"]


@pytest.fixture(scope="session")
def tgv_splitgauss_reference():
    import numpy as np
    d = np.load(os.path.join(ROOT, "tests", "golden", "tgv_splitgauss_reference.npz"))
    return d["header"], d["rows"]


@pytest.fixture(scope="session")
def tgv_oint_reference():
    import numpy as np
    d = np.load(os.path.join(ROOT, "tests", "golden", "tgv_oint_reference.npz"))
    return d["header"], d["rows"]
