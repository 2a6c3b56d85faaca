import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (REPO, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests of the engine")
    config.addinivalue_line("markers", "slow: full-size configuration, seconds to minutes")


@pytest.fixture(scope="session")
def oracle():
    """The CPU checker (built on first use)."""
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def engine_lib():
    """The engine's shared library, built in-tree if stale."""
    from geopvi_gb300 import build, _native
    build.build()
    return _native.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test on a machine without CUDA: run with -m 'not gpu'")
    return torch.device("cuda:0")
