"""Failure detection on the GPU without a fault: the tensor-core GEMM's
bounded mbarrier wait, on a barrier that nothing arrives on, gives up after
its poll limit and reports it through a device flag the host reads; the
same wait completes when the arrival comes; the context stays usable
afterwards (a torch kernel, the GEMM's status flag untouched).  The same for
the cell sort's single-pass scan: a tile whose predecessor never publishes
its sum stops waiting after its poll limit and says so."""
import pytest
import torch

from chimeracl_gb300 import _lib
from chimeracl_gb300._lib import call

pytestmark = pytest.mark.gpu

SPINS = 100000  # a few milliseconds of polls


def test_wait_gives_up_and_context_stays_usable(cuda):
    lib = _lib.load()
    flag = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    call("ccl_wait_probe", SPINS, 0, flag.data_ptr(), _lib.stream())
    torch.cuda.synchronize()
    assert int(flag.item()) == 1  # nothing arrived: the wait ran out
    call("ccl_wait_probe", SPINS, 1, flag.data_ptr(), _lib.stream())
    torch.cuda.synchronize()
    assert int(flag.item()) == 0  # the arrival completed the phase
    x = torch.arange(8, device="cuda", dtype=torch.float64)
    assert float((2 * x).sum()) == 56.0
    assert lib.ccl_dht_bf16x3_status(0) == 0
    assert lib.ccl_wait_probe(0, 0, flag.data_ptr(), None) == 1  # rejected, not launched


def test_scan_lookback_wait_gives_up(cuda):
    lib = _lib.load()
    flag = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    scratch = torch.zeros(8, dtype=torch.int32, device="cuda")
    call("ccl_scan_wait_probe", SPINS, 0, flag.data_ptr(), scratch.data_ptr(), _lib.stream())
    torch.cuda.synchronize()
    assert int(flag.item()) == 1  # the predecessor never published: the wait ran out
    assert int(scratch[6].item()) == 0  # its sum counted as zero
    call("ccl_scan_wait_probe", SPINS, 1, flag.data_ptr(), scratch.data_ptr(), _lib.stream())
    torch.cuda.synchronize()
    assert int(flag.item()) == 0
    assert int(scratch[6].item()) == 5  # the predecessor's inclusive prefix
    # the tile published its own inclusive prefix, 5 + 7, with flag 2
    assert int(scratch[2].item()) == 12 and int(scratch[3].item()) == 2
    x = torch.arange(8, device="cuda", dtype=torch.float64)
    assert float((2 * x).sum()) == 56.0
    assert lib.ccl_sort_status(0) == 0  # the probe reports through its own flag
    assert lib.ccl_scan_wait_probe(0, 0, flag.data_ptr(), scratch.data_ptr(), None) == 1
