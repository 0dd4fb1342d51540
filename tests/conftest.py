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


def rel(a, b):
    import numpy as np
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def make_pair(nx, ny, nzp, Lz=2.0, precision=0, cz=25, oz=5, Lx=1.0, Ly=1.0):
    """(GPU plan, oracle grid) for the same channel grid."""
    from oracle import oracle as O
    from specter_gb300 import api
    nz = nzp + cz
    plan = api.Plan((nx, ny, nz), (0, 0, cz), (0, 0, oz), (Lx, Ly, Lz), precision=precision)
    grid = O.Grid(nx, ny, nz, cz, oz, Lx, Ly, Lz)
    return plan, grid


def smooth_spectral(grid, rng, nmodes=5, kmax=3, amp=1.0):
    """Seeded smooth real field on the physical rows, transformed by the oracle's r2c."""
    import numpy as np
    x = 2 * np.pi * grid.Lx * np.arange(grid.nx) / grid.nx
    y = 2 * np.pi * grid.Ly * np.arange(grid.ny) / grid.ny
    Z, Y, X = np.meshgrid(grid.z, y, x, indexing="ij")
    r = np.zeros(grid.rshape)
    for _ in range(nmodes):
        kx, ky = rng.integers(-kmax, kmax + 1, 2)
        r += rng.standard_normal() * np.cos(kx * X / grid.Lx + ky * Y / grid.Ly + rng.uniform(0.3, 3.0) * Z + rng.uniform(0, 2 * np.pi))
    r[grid.nz - grid.cz:] = 0.0
    return grid.fftp3d_real_to_complex(r * amp)


@pytest.fixture(scope="session")
def channel_grid(oracle_mod):
    """64 x 64 x (65 + 25) channel, Lx = Ly = 2*pi, Lz = 2 (the plain-FP64 HD configuration)."""
    return oracle_mod.Grid(64, 64, 90, 25, 5, 1.0, 1.0, 2.0)
