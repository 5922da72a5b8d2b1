"""The coordinate push fused with the sort's first pass (ccl_push_x_keys +
ccl_index_sort_keyed) through the C ABI: its outputs are those of push_xyz
followed by the cell sort.

* FP64 against the oracle (push_xyz, index_and_sum_in_cell, sort of the
  reference's kernels): pushed coordinates, keys, counts, offsets, sort
  order and in-window count identical, on 16-byte-aligned arrays (vector
  path, a tail of odd length) and on misaligned ones (scalar path);
* FP32, plain and compensated coordinates: identical, bit for bit, to the
  separate calls (ccl_push_x / ccl_push_x_compensated, ccl_index_sort).
"""
import numpy as np
import pytest
import torch

from chimeracl_gb300 import _lib
from chimeracl_gb300._lib import CCL_F32, CCL_F64, call
from tests.test_gpu_kernels import S, dev, geom, host, oracle_sort, particles

pytestmark = pytest.mark.gpu
DT = 0.0217


def _bufs(n, g):
    C_ = (g["Nx"] - 1) * (g["Nr"] - 1)
    i32 = dict(dtype=torch.int32, device="cuda")
    wsb = _lib.sort_workspace_bytes(n, C_)
    return dict(indx=torch.empty(max(n, 1), **i32), cnt=torch.empty(C_ + 1, **i32),
                off=torch.empty(C_ + 2, **i32), srt=torch.empty(max(n, 1), **i32),
                nst=torch.empty(1, **i32), ws=torch.empty(wsb, dtype=torch.uint8, device="cuda"),
                wsb=wsb)


def _fused(dtype, n, d, g, lo=None, off=0):
    """push + keys, then the rest of the sort; `off` elements into each array
    (off = 1: nothing is 16-byte aligned)."""
    b = _bufs(n, g)
    P = lambda k: d[k].data_ptr() + off * d[k].element_size()  # noqa: E731
    lop = [P(k) for k in lo] if lo else [None] * 3
    call("ccl_push_x_keys", dtype, n, P("x"), P("y"), P("z"), *lop, P("px"), P("py"), P("pz"),
         P("g_inv"), DT, g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"],
         b["indx"].data_ptr(), b["cnt"].data_ptr(), b["ws"].data_ptr(), b["wsb"], S())
    call("ccl_index_sort_keyed", n, g["Nx"], g["Nr"], b["indx"].data_ptr(), b["cnt"].data_ptr(),
         b["off"].data_ptr(), b["srt"].data_ptr(), b["nst"].data_ptr(), b["ws"].data_ptr(),
         b["wsb"], S())
    torch.cuda.synchronize()
    return b


def _sort_out(b, n):
    return (host(b["indx"], np.uint32)[:n], host(b["cnt"], np.uint32), host(b["off"], np.uint32),
            host(b["srt"], np.uint32)[:n], int(host(b["nst"])[0]))


@pytest.mark.parametrize("n,Nx,Nr,off", [(0, 32, 8, 0), (1, 32, 8, 0), (7, 32, 8, 0),
                                         (100003, 96, 24, 0), (300000, 512, 64, 0),
                                         (20001, 96, 24, 1)])
def test_push_keys_fp64_matches_oracle(cuda, port, n, Nx, Nr, off):
    rng = np.random.default_rng(n + Nx + off)
    g = geom(Nx, Nr)
    p = particles(rng, n + off, g)
    d = {k: dev(v) for k, v in p.items()}
    b = _fused(CCL_F64, n, d, g, off=off)
    q = {k: v[off:].copy() for k, v in p.items()}
    port.push_xyz(q["x"], q["y"], q["z"], q["px"], q["py"], q["pz"], q["g_inv"], DT)
    for k in ("x", "y", "z"):
        np.testing.assert_array_equal(host(d[k])[off:], q[k], err_msg=k)
    oi, oc, oo, osr = oracle_sort(port, q, g)
    gi, gc, go, gsr, nst = _sort_out(b, n)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gc, oc)
    np.testing.assert_array_equal(go, oo)
    np.testing.assert_array_equal(gsr, osr)
    assert nst == int(oo[-2])


@pytest.mark.parametrize("compensated", [False, True])
def test_push_keys_fp32_equals_separate_calls(cuda, compensated):
    rng = np.random.default_rng(21 + compensated)
    g = geom(2048, 256, Xmin=-80.0, Xmax=0.0, Rmax=40.0)
    n = 1_000_003
    p = {k: v.astype(np.float32) for k, v in particles(rng, n, g).items()}
    lo = ("x_lo", "y_lo", "z_lo") if compensated else None
    if compensated:
        for c in "xyz":
            p[c + "_lo"] = (rng.uniform(-0.5, 0.5, n) * np.spacing(p[c])).astype(np.float32)
    a = {k: dev(v) for k, v in p.items()}
    s = {k: dev(v) for k, v in p.items()}
    b = _fused(CCL_F32, n, a, g, lo=lo)
    names = ("x", "y", "z") + (lo or ()) + ("px", "py", "pz", "g_inv")
    call("ccl_push_x_compensated" if compensated else "ccl_push_x", CCL_F32, n,
         *[s[k].data_ptr() for k in names], DT, S())
    r = _bufs(n, g)
    call("ccl_index_sort", CCL_F32, n, s["x"].data_ptr(), s["y"].data_ptr(), s["z"].data_ptr(),
         g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"], r["indx"].data_ptr(),
         r["cnt"].data_ptr(), r["off"].data_ptr(), r["srt"].data_ptr(), r["nst"].data_ptr(),
         r["ws"].data_ptr(), r["wsb"], S())
    torch.cuda.synchronize()
    for k in ("x", "y", "z") + (lo or ()):
        np.testing.assert_array_equal(host(a[k]).view(np.uint32), host(s[k]).view(np.uint32),
                                      err_msg=k)
    for u, v in zip(_sort_out(b, n), _sort_out(r, n)):
        np.testing.assert_array_equal(u, v)
