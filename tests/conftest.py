import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def stpgb():
    import superterrainplus_gb300 as m
    m.lib()
    return m


@pytest.fixture(scope="session")
def dev(stpgb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return stpgb.DeviceOps()


@pytest.fixture
def shf_path(dev):
    """Sets the filter's process-wide path (stpgb_shf_set_path) for one test, then back to 0."""
    yield dev.shf_set_path
    dev.shf_set_path(0)
