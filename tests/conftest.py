import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (run with -m gpu)')


@pytest.fixture(scope='session')
def oracle():
    import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope='session')
def pkg():
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope='session')
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail('CUDA is required for -m gpu tests')
    return torch
