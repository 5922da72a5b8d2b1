"""ccl_index_sort_noalloc (the cell sort with its workspace in a static
device array) against ccl_index_sort with a caller-owned workspace, through
the C ABI.  Collected last (file name) so that it also runs after every
other test in the same process."""
import os

import numpy as np
import pytest

from chimeracl_gb300 import _lib
from chimeracl_gb300._lib import CCL_F32, CCL_F64


def _geom(Nx, Nr, Xmin=-20.0, Xmax=0.0, Rmax=8.0):
    dx = (Xmax - Xmin) / (Nx - 1)
    dr = Rmax / (Nr - 1.5)
    return dict(Nx=Nx, Nr=Nr, Xmin=Xmin, dx_inv=1.0 / dx, Rmin=-0.5 * dr, dr_inv=1.0 / dr,
                Xmax=Xmax, Rmax=Rmax)


def test_oversize_rejected_without_launch():
    """Too large for the 9 MiB scratch: an error, before any CUDA call."""
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    g = _geom(4097, 2049)
    rc = lib.ccl_index_sort_noalloc(CCL_F64, 1000, None, None, None, g["Nx"], g["Xmin"],
                                    g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"], None, None,
                                    None, None, None, None)
    assert rc == 4
    assert b"static scratch" in lib.ccl_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [CCL_F64, CCL_F32])
def test_noalloc_sort_matches_workspace_sort(cuda, dtype):
    import torch
    rng = np.random.default_rng(17 + dtype)
    g = _geom(512, 96)
    n = 400_000
    L = g["Xmax"] - g["Xmin"]
    x = rng.uniform(g["Xmin"] - 0.1 * L, g["Xmax"] + 0.1 * L, n)
    r = rng.uniform(0, g["Rmax"] * 1.1, n)
    th = rng.uniform(0, 2 * np.pi, n)
    ft = np.float64 if dtype == CCL_F64 else np.float32
    pos = [torch.from_numpy(a.astype(ft)).cuda() for a in (x, r * np.cos(th), r * np.sin(th))]
    C = (g["Nx"] - 1) * (g["Nr"] - 1)
    i32 = dict(dtype=torch.int32, device="cuda")

    def outputs():
        return [torch.empty(n, **i32), torch.empty(C + 1, **i32), torch.empty(C + 2, **i32),
                torch.empty(n, **i32), torch.empty(1, **i32)]

    geo = (g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"])
    ref = outputs()
    wsb = _lib.sort_workspace_bytes(n, C)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.call("ccl_index_sort", dtype, n, *[p.data_ptr() for p in pos], *geo,
              *[t.data_ptr() for t in ref], ws.data_ptr(), wsb, _lib.stream())
    torch.cuda.synchronize()
    for _ in range(2):  # two calls in a row: the static scratch is reused
        got = outputs()
        for t in got:
            t.fill_(-1)
        _lib.call("ccl_index_sort_noalloc", dtype, n, *[p.data_ptr() for p in pos], *geo,
                  *[t.data_ptr() for t in got], _lib.stream())
        torch.cuda.synchronize()
        for a, b in zip(ref, got):
            assert torch.equal(a, b)
    assert 0 < int(ref[4][0]) < n
