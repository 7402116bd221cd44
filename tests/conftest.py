import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG = REPO / "mosaic-art-rust_gb300"
for p in (str(PKG), str(REPO)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def built():
    """Build the in-tree libraries (cached by timestamps) and the oracle."""
    from mosaic_gpu import build as b

    import oracle.binding as ob

    paths = b.build()
    ob.build_oracle()
    return paths


@pytest.fixture(scope="session")
def orc(built):
    import oracle.binding as ob

    ob.lib()
    return ob


@pytest.fixture(scope="session")
def ctx(built):
    from mosaic_gpu import _capi as capi

    c = capi.Context(0)
    yield c
    c.close()
