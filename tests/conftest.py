import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libspecter_gpu.so")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def channel_grid(oracle_mod):
    """64 x 64 x (65 + 25) channel, Lx = Ly = 2*pi, Lz = 2 (the plain-FP64 HD configuration)."""
    return oracle_mod.Grid(64, 64, 90, 25, 5, 1.0, 1.0, 2.0)
