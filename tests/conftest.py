import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (CUDA device 0)")


@pytest.fixture(scope="session")
def built():
    """Compile the CUDA library and the oracle once per session."""
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def model_root(tmp_path_factory):
    return tmp_path_factory.mktemp("models")
