"""Test configuration: markers and loaders for the package and the oracle."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "sc17-born_gb300")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def load_package():
    """Imports sc17-born_gb300/ as module ``born_gb300``."""
    if "born_gb300" in sys.modules:
        return sys.modules["born_gb300"]
    spec = importlib.util.spec_from_file_location(
        "born_gb300", os.path.join(PKG_DIR, "__init__.py"),
        submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["born_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def born():
    mod = load_package()
    mod.build()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def po():
    import pyoracle
    pyoracle.build_port()
    return pyoracle
