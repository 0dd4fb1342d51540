"""The C-ABI library loads without a GPU and exports every function include/specter_gpu.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "specter_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(specter_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from specter_gb300 import build
    build.build()
    return ctypes.CDLL(build.LIB)


def test_header_parses():
    names = declared_functions()
    assert "specter_plan_create" in names and "specter_solver_step" in names
    assert len(names) >= 40


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from specter_gb300._lib import EXPORTS
    assert set(EXPORTS) == set(declared_functions())


def test_errors_without_gpu_are_loud(lib):
    """With no CUDA device, plan creation fails with SPECTER_ERR_CUDA (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from specter_gb300 import api, SpecterError
    with pytest.raises(SpecterError) as e:
        api.Plan((16, 16, 58))
    assert e.value.code == 5


def test_version(lib):
    lib.specter_version.restype = ctypes.c_int
    assert lib.specter_version() >= 100
