import os
import sys

# The oracle's OpenMP threads would otherwise spin between its short kernels
# and compete with numpy's BLAS threads for the cores (12x slower oracle
# steps on a 512 x 64 grid); the policy has to be set before the first
# library that uses OpenMP (torch, the oracle) is loaded.
os.environ.setdefault("OMP_WAIT_POLICY", "passive")

import pytest  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from chimeracl_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)


@pytest.fixture(scope="session")
def port():
    from oracle.kernels import PortKernels
    return PortKernels()
