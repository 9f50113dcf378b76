import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def dpg_lib():
    """libdpg.so, built in-tree on first use."""
    from dynoplan_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build_library()
    return _lib.load()
