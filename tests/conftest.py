import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA library, built in-tree; GPU tests fail loudly if it cannot load."""
    from sph_seepage_flows_gb300 import build, capi
    build.build_library()
    lib = capi.load()
    if lib.sf_device_count() <= 0:
        pytest.fail("no CUDA device visible to libsf_gb300.so")
    return lib


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
