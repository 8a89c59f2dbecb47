import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle and the native libraries once per session."""
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    from maplab_gb300 import build
    build.build()
    yield
