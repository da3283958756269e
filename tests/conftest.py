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
    """Build libtbfs.so and the oracle in-tree (no-op when up to date)."""
    from turbobfs_gb300 import build

    build.build()
    build.build_oracle()


@pytest.fixture(scope="session")
def gpu_available(_built):
    from turbobfs_gb300 import device_count

    if device_count() < 1:
        pytest.fail("GPU test collected on a machine without a visible CUDA device")
    return True
