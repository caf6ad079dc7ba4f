import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle (and the library when nvcc is present) once per session."""
    from oracle import build as ob

    ob.build_oracle()
    try:
        ob.build_reference()
    except RuntimeError:
        pass
    from trayracer_gb300 import build as tb

    try:
        tb.build()
    except RuntimeError:
        pass
    yield
