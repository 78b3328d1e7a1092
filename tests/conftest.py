import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU check")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    cache = {}

    def load(name):
        if name not in cache:
            cache[name] = dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))
        return cache[name]

    return load


_REPORT = []


@pytest.fixture(scope="session")
def parity_report():
    """Collects (case, iterations, field, relative L2) rows; written as JSON lines to
    $GRAPTOR_PARITY_REPORT at the end of the session when that variable is set."""
    yield _REPORT.append


def pytest_sessionfinish(session, exitstatus):
    path = os.environ.get("GRAPTOR_PARITY_REPORT")
    if path and _REPORT:
        import json
        with open(path, "w") as f:
            for row in _REPORT:
                f.write(json.dumps(row) + "\n")
