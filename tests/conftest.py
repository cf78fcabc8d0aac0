import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: longer CPU-side checks")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def pfs_lib():
    """The CUDA library, built in-tree if needed. No fallback: failure to build or load fails the test."""
    from probabilistic_fluid_simulation_gb300 import build, fluid
    build.build()
    fluid.lib()
    return fluid


@pytest.fixture(scope="session")
def cuda_device(pfs_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a visible CUDA device")
    return torch.device("cuda:0")
