import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_pkg():
    """Imports the package directory `mpi-rockstar_gb300` as mpi_rockstar_gb300."""
    if "mpi_rockstar_gb300" in sys.modules:
        return sys.modules["mpi_rockstar_gb300"]
    d = os.path.join(ROOT, "mpi-rockstar_gb300")
    spec = importlib.util.spec_from_file_location(
        "mpi_rockstar_gb300", os.path.join(d, "__init__.py"), submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules["mpi_rockstar_gb300"] = m
    spec.loader.exec_module(m)
    return m


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def rk():
    m = load_pkg()
    m.build()
    return m


@pytest.fixture(scope="session")
def oracle():
    from oracle import restatement
    restatement.build()
    return restatement
