import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "gamil-dycore_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the native library")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def native():
    """Build (if needed) and load libgdc.so; the CUDA path has no fallback."""
    build = __import__("build")
    build.build()
    import gdc
    return gdc.lib()
