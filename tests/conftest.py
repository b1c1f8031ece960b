import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REFERENCE = "/root/reference"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "slow: long-running oracle comparison")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU visible")
    from pis_gb300 import build
    build.build()
    from pis_gb300 import _ffi
    return _ffi.lib()


def reference_file(*parts):
    p = os.path.join(REFERENCE, *parts)
    if not os.path.exists(p):
        pytest.skip("reference sources not mounted")
    return p
