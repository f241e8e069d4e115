import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built engine")


@pytest.fixture(scope="session")
def engine():
    """One engine handle on cuda:0 for the whole GPU session (built in-tree first)."""
    import torch

    from eating_one_gb300.build import build
    from eating_one_gb300.engine import Engine

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    build()
    e = Engine(0)
    yield e
    e.close()
