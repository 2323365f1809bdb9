import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "latticemodels.jl_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the lmgpu kernels)")


@pytest.fixture(scope="session")
def lib():
    import lmgpu._lib as L
    return L.load()
