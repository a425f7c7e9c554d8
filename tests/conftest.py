"""Test configuration: the package and the oracle on sys.path, the gpu marker.

GPU tests (``-m gpu``) call the CUDA engine through its C ABI and compare it
with the oracle; everything else runs on the CPU.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "treeamr.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda_lib():
    """The built engine; GPU tests fail loudly (never fall back) when it is
    missing."""
    if not gpu_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    from treeamr import _native
    _native.build()
    return _native.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle.lib()
