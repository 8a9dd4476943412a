import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def lib_path():
    from globillum_gb300 import build
    return build.build_lib()


@pytest.fixture(scope="session")
def gpu_ctx(lib_path):
    from globillum_gb300 import gbpt
    ctx = gbpt.Context(0)
    yield ctx
    ctx.close()
