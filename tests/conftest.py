import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def golden_paths():
    d = os.path.join(ROOT, "tests", "golden")
    return sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith(".npz"))
