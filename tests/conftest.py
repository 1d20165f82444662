import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built libemp_gpu.so')


@pytest.fixture(scope='session')
def peg_arr():
    return np.load(os.path.join(GOLDEN, '51peg_rv.npz'))['data']


@pytest.fixture(scope='session')
def kat():
    return np.load(os.path.join(GOLDEN, 'logpost_kat.npz'))


@pytest.fixture(scope='session')
def lib():
    """The native library, built in-tree if missing (nvcc cross-compiles)."""
    from astroemperor_gb300 import build, _native
    if not build.up_to_date():
        build.build()
    return _native.load()


@pytest.fixture(scope='session')
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return torch.device('cuda:0')
