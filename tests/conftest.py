import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libbvhgpu.so and the oracle once (no-op when up to date)."""
    from bvhraytracer_gb300 import build as B
    from oracle import build_oracle
    B.build()
    build_oracle.build()
