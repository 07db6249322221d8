import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "dials-metal_gb300"):
    path = os.path.join(REPO, sub)
    if path not in sys.path:
        sys.path.insert(0, path)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """The oracle is compiled on first use; the CUDA library by build()."""
    import oracle
    oracle.lib()
