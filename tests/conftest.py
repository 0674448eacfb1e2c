import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure)."""
    return graft.load_oracle()


@pytest.fixture(scope="session")
def nlpkg():
    """The product package (libnlgpu.so must be built)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("nl_gb300_build", os.path.join(graft.PKG_DIR, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    return graft.load_package()
