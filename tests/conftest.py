import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmdt_gpu.so")


@pytest.fixture(scope="session")
def built_lib():
    """Builds the CUDA engine library in-tree (nvcc cross-compiles without a GPU)."""
    from md_tian2_gb300.build import build
    return build()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle
