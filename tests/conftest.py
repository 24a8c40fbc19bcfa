import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    # the library must be the compute path: loading it is part of the test
    from nrpytutorial_gb300 import _lib
    _lib.load()
    return torch.device("cuda:0")


@pytest.fixture(params=["point", "staged", "fused"])
def bssn_kernels(request, cuda):
    """Runs a BSSN test once per kernel family (nrgpu_set_bssn_kernels): the
    point kernels, the shared-memory staged kernels, and the staged kernels
    with Ricci fused into the MoL step's RHS kernel.  Afterwards the library's
    device status word must be clear (no bounded wait gave up)."""
    import nrpytutorial_gb300 as pkg
    prev = pkg.set_bssn_kernels(request.param)
    try:
        yield request.param
    finally:
        pkg.set_bssn_kernels(prev)
    assert pkg.device_status() == 0
