import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cfd-lite_gb300")
for p in (ROOT, PKG, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libcfdgpu.so")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the product library and the oracle once per session (both are
    cheap no-ops when up to date)."""
    import build as pkg_build  # cfd-lite_gb300/build.py
    import oracle_lib
    pkg_build.build()
    oracle_lib.build_oracle()
    yield


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture
def need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")
