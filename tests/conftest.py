import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT / "finiteelementcontainers.jl_gb300"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libfec_gb300.so")


@pytest.fixture(scope="session")
def fec():
    """The product package with its library built (builds on first use)."""
    import fec_gb300
    from fec_gb300 import build
    if not build.LIB.exists():
        build.build()
    fec_gb300.load_library()
    return fec_gb300


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.lib()
    return oracle
