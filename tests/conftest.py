import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build
    build.build()
    from oracle import fluid_c
    return fluid_c


@pytest.fixture(scope="session")
def tg():
    """The package with its CUDA library built and loaded (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tinyfluids_gb300 import build
    build.build()
    import tinyfluids_gb300
    tinyfluids_gb300._lib.load()
    return tinyfluids_gb300
