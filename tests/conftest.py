import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Builds (or reuses) libvfs_cuda.so and the oracle before any test runs."""
    from vkfluidsim_gb300.build import build_all

    build_all()


@pytest.fixture(autouse=True)
def _require_device(request):
    if request.node.get_closest_marker("gpu") is None:
        return
    from vkfluidsim_gb300 import load_library

    if load_library().vfs_device_count() < 1:
        pytest.skip("no CUDA device visible")
