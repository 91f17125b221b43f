import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "mc-mpi_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def import_package():
    """Import the mc-mpi_gb300 directory as the package `mc_mpi_gb300`."""
    if "mc_mpi_gb300" in sys.modules:
        return sys.modules["mc_mpi_gb300"]
    spec = importlib.util.spec_from_file_location(
        "mc_mpi_gb300", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["mc_mpi_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def mcg():
    return import_package()


@pytest.fixture(scope="session")
def built():
    """Build the library and the strict tables once per session."""
    import_package()
    from mc_mpi_gb300 import build as B
    B.build()
    return B


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O
