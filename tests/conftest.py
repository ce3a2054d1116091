import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def fluid():
    """The package with its CUDA library built and loaded."""
    import fluid2d_gb300 as pkg
    from fluid2d_gb300 import build_lib

    build_lib.build()
    pkg.load()
    return pkg


@pytest.fixture(scope="session")
def wl():
    from fluid2d_gb300 import workloads

    return workloads
