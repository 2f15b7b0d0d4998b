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
    config.addinivalue_line("markers", "timeout(seconds): per-test limit (pytest-timeout, when installed)")


def pytest_collection_modifyitems(config, items):
    # a per-test limit on the GPU tests (when pytest-timeout is installed): a solve that stops
    # converging ends the run instead of holding it (the thread method also ends a test that
    # waits inside the library, where no signal reaches the interpreter)
    if not config.pluginmanager.hasplugin("timeout"):
        return
    for item in items:
        if item.get_closest_marker("gpu") and not item.get_closest_marker("timeout"):
            item.add_marker(pytest.mark.timeout(900, method="thread"))


@pytest.fixture(scope="session")
def dcgpu_lib():
    """Build (if needed) and load libdcgpu; returns the dcgpu binding module."""
    import __graft_entry__ as g
    g.build()
    import dcgpu
    dcgpu.load_library()
    return dcgpu
