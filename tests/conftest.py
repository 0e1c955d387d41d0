import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def ora():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def built():
    from tbslas_gb300 import build
    build.build()
    from tbslas_gb300 import capi
    return capi.lib()


@pytest.fixture(scope="session")
def ctx(built):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from tbslas_gb300 import Context
    c = Context(0)
    yield c
    assert c.check() == 0
    c.close()
