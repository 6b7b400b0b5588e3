import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def oracle_built():
    """Compile the oracle (C restatement) once per session."""
    import pyoracle

    pyoracle.build()
    return True


@pytest.fixture(scope="session")
def gpu():
    """Build (if stale) and load the CUDA library; GPU tests need a GB300."""
    from ffea_ci_demo_gb300 import build, lib

    build.build()
    return lib.load()
