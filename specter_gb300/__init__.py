"""specter_gb300: SPECTER's per-RK-stage hot path (FC-Gram transforms, pseudo-spectral
nonlinear terms, wall projection, RK update) as hand-written sm_103a CUDA behind a C ABI.

The compute lives in libspecter_gpu.so (include/specter_gpu.h); this package is its
host-side mirror of the reference's fftp / pseudo / boundary interfaces.  Importing it
does not touch the GPU; the library is loaded on first use.
"""
from ._lib import SpecterError  # noqa: F401
from . import api  # noqa: F401

__version__ = "0.1.0"
