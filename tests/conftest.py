import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "trekis-3_gb300", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) device")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle_py
    return oracle_py.load()


@pytest.fixture(scope="session")
def gpu_lib():
    from trekis import abi, build
    build.build_library()
    lib = abi.load()
    assert lib.trekis_device_ok() == 1, "a GPU test ran without a usable sm_103a device"
    return lib


def copy_tables(t, o, w):
    """Load GPU-built tables into the oracle so both MC implementations run on
    identical data (the tables themselves are compared separately)."""
    import __graft_entry__ as g
    g._copy_tables(t, o, w)
