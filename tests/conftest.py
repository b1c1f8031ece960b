import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# The reference crate's sources, when mounted: tests that read its example files directly take the
# directory from PIS_REFERENCE_DIR and skip when it is unset (the golden fixtures carry the known
# answers taken from those files, with their SHA-256, for machines without them).
REFERENCE = os.environ.get("PIS_REFERENCE_DIR", "")


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
    if not REFERENCE:
        pytest.skip("PIS_REFERENCE_DIR is not set")
    p = os.path.join(REFERENCE, *parts)
    if not os.path.exists(p):
        pytest.skip("reference sources not mounted")
    return p
