import os
import sys
import pathlib

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402

graft.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library through its C ABI)")


@pytest.fixture(scope="session")
def mg():
    return graft.load_package()


@pytest.fixture(scope="session")
def orc():
    return graft.load_oracle()


@pytest.fixture(scope="session")
def lib(mg):
    lib_build = graft._build_module(graft.PKG_DIR / "build.py", "_mavi_build")
    lib_build.build()
    return mg.load_library()
