import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the kernels through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def native_build():
    """Compile the native libraries (incremental; nvcc cross-compiles without a GPU)."""
    from midsx_gb300 import build
    build.build()
    return True


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "hvl_reference.json")) as f:
        return json.load(f)
