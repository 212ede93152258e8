import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the native CUDA path")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def owm():
    """The package with its native library built (compiles on first use)."""
    from fastowm_gb300 import build as b

    b.build()
    import fastowm_gb300 as F

    F.lib()
    return F


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build(ref=False)
    return O


@pytest.fixture(scope="session")
def ctx(owm):
    c = owm.Context(0)
    yield c
    c.close()
