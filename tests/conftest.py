import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def lib():
    """The in-tree librustracer_cuda.so, built if stale."""
    from rustracer_gb300 import build as b

    b.build()
    from rustracer_gb300 import _abi

    return _abi.load()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build()
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def gpu(lib):
    """Fails (does not skip) when a GPU test runs without a device: the kernels have no fallback."""
    n = lib.rt_device_count()
    if n < 1:
        pytest.fail("a gpu-marked test ran without a visible CUDA device")
    return n
