"""Test configuration: the `gpu` marker and session fixtures that build the
oracle (gcc) and the engine library (nvcc, sm_103a)."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; calls the engine through its C ABI")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def engine():
    from opendxmc_gb300 import build

    build.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G

    return G


@pytest.fixture(scope="session")
def gpu(engine):
    """The GPU tests fail (never skip) when no device is visible."""
    n = engine.device_count()
    assert n > 0, "no CUDA device visible: the -m gpu tests need a GPU"
    return engine
