import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "itensornetworks.jl_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libgbtn.so built for sm_103a")


@pytest.fixture(scope="session")
def lib_built():
    from gbtn import build

    build.build()
    return build.LIB_PATH
