import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libxr.so and the oracle once per session (in-tree, incremental)."""
    from xvk_ray_gb300 import _build

    _build.build_library()
    _build.build_oracle()
    yield
