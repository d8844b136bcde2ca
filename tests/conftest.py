"""pytest configuration: the ``gpu`` marker and import paths.

Tests marked ``gpu`` need a CUDA device and the built library; everything
else runs on the CPU (oracle, host logic, file formats, symbol exports)."""
import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
PKG = os.path.join(ROOT, "cufim-nvlink_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def built_library():
    """Builds the solver library (sm_103a) once per session and returns its path."""
    import build as pkg_build
    return pkg_build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as obuild
    obuild.build_oracle()
    from oracle import oracle
    return oracle
