import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")
    config.addinivalue_line("markers", "slow: full-size volumes")


@pytest.fixture(scope="session")
def fclib():
    """The product library, built in-tree if needed."""
    from fourierconvolutioncudalib_gb300 import build as fcbuild
    import fourierconvolutioncudalib_gb300 as fc

    fcbuild.build()
    return fc.load_library()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.build_oracle()
    return oracle


@pytest.fixture(scope="session")
def cuda(fclib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
