import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, 'oracle'), os.path.join(ROOT, 'tests', 'golden')):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built library')
    config.addinivalue_line('markers', 'slow: long-running statistical test')


@pytest.fixture(scope='session')
def lib():
    from pyxopto_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from pyxopto_gb300 import build
        build.build()
    return _lib.load()


@pytest.fixture(scope='session')
def oracle():
    import mcoracle
    mcoracle.build()
    return mcoracle


@pytest.fixture(scope='session')
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return torch
