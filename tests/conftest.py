import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pseudotransientdiffusion.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libptd.so kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libptd.so (nvcc cross-compiles without a GPU) and the CPU oracle once."""
    import build as _build
    from oracle import oracle as _oracle

    _build.build()
    _oracle.build()
    yield
