"""Shared test set-up: import paths, markers and library builds."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "procedural-universe_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Builds the product library and the oracle once per session if stale."""
    import nb_build as pkg_build  # procedural-universe_gb300/nb_build.py
    from oracle import oracle as O

    pkg_build.build()
    O.build()
    yield
