import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    import axisem_gb300.build as b
    from axisem_gb300 import _abi

    b.build()
    return _abi.load_library()


@pytest.fixture(scope="session")
def gpu_lib(lib):
    n = lib.axg_device_count()
    assert n >= 1, "GPU tests need a CUDA device; the library has no CPU fallback"
    return lib


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.build()
    return oracle
