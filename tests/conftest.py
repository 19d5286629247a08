import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_py
    oracle_py.build()
    return oracle_py


@pytest.fixture(scope="session")
def engine():
    """The engine library, built in-tree; on a GPU machine its load is part of what is tested."""
    from wobtoolbox_gb300 import build as b
    b.build()
    import wobtoolbox_gb300 as wob
    wob.load()
    return wob


@pytest.fixture(scope="session")
def cuda(engine):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("tests marked gpu need a CUDA device")
    torch.cuda.set_device(0)
    return torch
