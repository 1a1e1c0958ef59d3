import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the encoder kernels)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def reference():
    import pyoracle
    if not pyoracle.Reference.available():
        pytest.skip("the reference encoder was not compiled here (its sources are absent)")
    return pyoracle.Reference()


@pytest.fixture(scope="session")
def lib():
    """The GPU library, built on demand."""
    import s2tc_gb300
    from s2tc_gb300 import build
    if not s2tc_gb300.LIB_PATH.exists():
        build.build_library()
    return s2tc_gb300.load()
