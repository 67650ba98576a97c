import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def thmm():
    import parallel_tree_hmm_gb300

    return parallel_tree_hmm_gb300


@pytest.fixture(scope="session")
def gpu(thmm):
    if not thmm.available():
        pytest.skip("no CUDA device")
    return thmm
