import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")


def _package():
    import __graft_entry__ as ge
    return ge._package()


@pytest.fixture(scope="session")
def pkg():
    return _package()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def wl(pkg):
    return pkg.workloads


@pytest.fixture(scope="session")
def potentials(tmp_path_factory, wl):
    d = tmp_path_factory.mktemp("pot")
    return {
        "fe": wl.write_setfl(str(d / "fe.setfl"), wl.PotentialSpec(n_ele=1, seed=7)),
        "fecuni": wl.write_setfl(str(d / "fecuni.setfl"), wl.PotentialSpec(n_ele=3, seed=5)),
    }


@pytest.fixture(scope="session")
def gpu_lib(pkg):
    """The CUDA library, built for sm_103a; GPU tests fail (not skip) when it cannot be built."""
    pkg.build.build()
    return pkg.load_library()
