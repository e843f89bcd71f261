import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gene-sequences-de-redundancy_gb300")
for p in (PKG, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: longer CPU-side case")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the library and the oracle once per session (incremental)."""
    import build as pkg_build  # gene-sequences-de-redundancy_gb300/build.py

    pkg_build.build()
    import oracle_binding

    oracle_binding.build()
    yield
