import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "dune-copasi_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU-only test")


@pytest.fixture(scope="session")
def dcgpu_lib():
    """Build (if needed) and load libdcgpu; returns the dcgpu binding module."""
    import __graft_entry__ as g
    g.build()
    import dcgpu
    dcgpu.load_library()
    return dcgpu
