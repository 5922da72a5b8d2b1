"""Determinism and order of the deposits, through the C ABI: the same sorted
particles deposited twice give bitwise the same charge and current (no
atomics, nothing depends on scheduling); a random permutation of the
particles' storage order -- the cell sort then lists each cell's particles
in another order -- changes the FP64 deposit only as the oracle's deposit
of the permuted particles changes (bit for bit), and both precisions only
by rounding (1e-13 of the deposited magnitude in FP64, 1e-5 in FP32)."""
import numpy as np
import pytest
import torch

from chimeracl_gb300._lib import CCL_F32, CCL_F64, PP, call
from tests.test_gpu_kernels import S, dev, geom, host, oracle_sort, particles

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _release_uploads():
    """The uploads that dev() keeps alive are released after each test."""
    yield
    import tests.test_gpu_kernels as k
    torch.cuda.synchronize()
    k._KEEP.clear()


def _deposit(dtype, M, vec, p, off, srt, g):
    """Deposit into zeroed fields on the device; host copies of the fields."""
    real = np.float64 if dtype == CCL_F64 else np.float32
    names = ["J" + c for c in "xyz"] if vec else ["rho"]
    order = [n + "_m" + str(m) for m in range(M + 1) for n in names]
    shape = (g["Nr"], g["Nx"])
    d = {k: torch.zeros(shape, dtype=torch.float64 if real is np.float64 else torch.float32,
                        device="cuda") if k.endswith("_m0") else
         torch.zeros(shape, dtype=torch.complex128 if real is np.float64 else torch.complex64,
                     device="cuda") for k in order}
    pd = {k: dev(v.astype(real)) for k, v in p.items()}
    srt_d, off_d = dev(srt), dev(off)
    args = (g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"])
    if vec:
        call("ccl_deposit_vector", dtype, M, srt_d.data_ptr(), off_d.data_ptr(),
             pd["x"].data_ptr(), pd["y"].data_ptr(), pd["z"].data_ptr(), pd["px"].data_ptr(),
             pd["py"].data_ptr(), pd["pz"].data_ptr(), pd["g_inv"].data_ptr(), pd["w"].data_ptr(),
             -1, *args, PP([d[k] for k in order]), S())
    else:
        call("ccl_deposit_scalar", dtype, M, srt_d.data_ptr(), off_d.data_ptr(),
             pd["x"].data_ptr(), pd["y"].data_ptr(), pd["z"].data_ptr(), pd["w"].data_ptr(),
             -1, *args, PP([d[k] for k in order]), S())
    torch.cuda.synchronize()
    return {k: host(v) for k, v in d.items()}


def _oracle_deposit(port, M, vec, p, off, srt, g):
    names = ["J" + c for c in "xyz"] if vec else ["rho"]
    order = [n + "_m" + str(m) for m in range(M + 1) for n in names]
    out = {k: np.zeros((g["Nr"], g["Nx"]), np.float64 if k.endswith("_m0") else np.complex128)
           for k in order}
    nxnr4 = (g["Nr"]) // 2 * (g["Nx"]) // 2
    if vec:
        port.depose_vector(M, nxnr4, srt, p["x"], p["y"], p["z"], p["px"], p["py"], p["pz"],
                           p["g_inv"], p["w"], off, -1, g["Nx"], g["Xmin"], g["dx_inv"],
                           g["Nr"], g["Rmin"], g["dr_inv"], [out[k] for k in order])
    else:
        port.depose_scalar(M, nxnr4, srt, p["x"], p["y"], p["z"], p["w"], off, -1, g["Nx"],
                           g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"],
                           [out[k] for k in order])
    return out


@pytest.mark.parametrize("dtype", [CCL_F64, CCL_F32])
@pytest.mark.parametrize("vec", [False, True])
def test_deposit_deterministic_and_order_independent(cuda, port, dtype, vec):
    M = 1
    rng = np.random.default_rng(70 + 2 * vec + dtype)
    g = geom(160, 40)
    p = particles(rng, 60000, g)
    if dtype == CCL_F32:  # FP32 inputs, exactly representable in both forms
        p = {k: v.astype(np.float32).astype(np.float64) for k, v in p.items()}
    _, _, off, srt = oracle_sort(port, p, g)
    a = _deposit(dtype, M, vec, p, off, srt, g)
    b = _deposit(dtype, M, vec, p, off, srt, g)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)  # run twice: same bits

    perm = rng.permutation(p["x"].size)
    q = {k: v[perm].copy() for k, v in p.items()}
    _, _, offq, srtq = oracle_sort(port, q, g)
    np.testing.assert_array_equal(offq, off)  # same cells, other order within them
    c = _deposit(dtype, M, vec, q, offq, srtq, g)
    if dtype == CCL_F64:
        ref = _oracle_deposit(port, M, vec, q, offq, srtq, g)
        for k in c:
            np.testing.assert_array_equal(c[k], ref[k], err_msg=k)
    tol = 1e-13 if dtype == CCL_F64 else 1e-5
    for k in c:
        scale = np.abs(a[k]).max()
        assert scale > 0, k
        err = np.abs(c[k].astype(np.complex128) - a[k].astype(np.complex128)).max() / scale
        assert err <= tol, (k, err)
