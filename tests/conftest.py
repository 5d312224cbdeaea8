import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmgr_gpu.so")


@pytest.fixture
def oracle_cr_erf():
    """The oracle with the correctly rounded erff the GPU's FP64 mode uses (the
    reference's erff difference cancels, so parity needs the same erff)."""
    import oracle
    oracle.set_erf_mode(1)
    yield
    oracle.set_erf_mode(0)


@pytest.fixture(scope="session")
def gpu_lib():
    """libmgr_gpu.so with a visible device; GPU tests fail (not skip) without them."""
    from magritte_gb300 import _abi
    lib = _abi.load()
    assert _abi.device_count() > 0, "no CUDA device visible"
    return lib
