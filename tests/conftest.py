import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile the native library and the oracle once per session (cached by mtime)."""
    from opencloth_gb300.build import build

    import oracle

    build()
    oracle.build(reference=True)
    yield
