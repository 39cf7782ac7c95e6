import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def golden_names():
    """Sampling fixtures (refsample_random.npz holds reference samples only)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN_DIR) if f.endswith(".npz") and not f.startswith("refsample_"))


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN_DIR
