import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs on the GB300 box")


@pytest.fixture(scope="session")
def rt():
    import __graft_entry__ as g

    g.build()
    import raytracergpu_mastersproject_gb300 as rt

    return rt


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a host without CUDA")
    torch.cuda.set_device(0)
    return torch
