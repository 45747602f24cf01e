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


# worst errors of the parity tests at the stated benchmark configurations, printed after the run
_PARITY_REPORT = []


@pytest.fixture(scope="session")
def parity_report():
    """report(name, value, bar): records a measured error next to its bar for the end-of-run summary."""
    def report(name, value, bar):
        _PARITY_REPORT.append((name, float(value), float(bar)))
    return report


def pytest_terminal_summary(terminalreporter, exitstatus, config):
    if _PARITY_REPORT:
        terminalreporter.write_sep("-", "parity at the stated configurations (worst relative error / bar)")
        for name, v, bar in _PARITY_REPORT:
            terminalreporter.write_line(f"{name:60s} {v:.3e} / {bar:.0e}")
