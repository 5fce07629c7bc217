import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def built_lib():
    """Builds libhdgpu.so (cross-compiles without a GPU) once per session."""
    from hausdorffdistance_gb300 import build
    return build.build_lib()


@pytest.fixture(scope="session")
def engine(built_lib):
    import hausdorffdistance_gb300 as hd
    e = hd.Engine(device=0)
    yield e
    e.close()
