"""The BF16x3 tensor-core Hankel GEMM (tcgen05) against an FP64 product of
the same FP32 operands.  BF16x3 keeps about 16 mantissa bits per product
and accumulates in FP32: the bar is 1e-4 of the result's largest magnitude
(measured errors are ~1e-5)."""
import numpy as np
import pytest
import torch

from chimeracl_gb300 import _lib
from chimeracl_gb300._lib import CCL_F32, CCL_F64, PP, call, ints, longs

pytestmark = pytest.mark.gpu
TOL = 1e-4


def prepare(A64, dtype=CCL_F64):
    m, k = A64.shape
    import ctypes
    nb = ctypes.c_size_t(0)
    call("ccl_dht_bf16x3_prepare_bytes", m, k, ctypes.byref(nb))
    out = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    src = torch.from_numpy(A64 if dtype == CCL_F64 else A64.astype(np.float32)).cuda()
    call("ccl_dht_bf16x3_prepare", dtype, src.data_ptr(), m, k, out.data_ptr(), nb.value,
         _lib.stream())
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("m,k,ncols,ldx,cplx_,beta", [
    (255, 255, 4096, 4096, 1, 0.0), (255, 255, 2048, 2048, 0, 0.0), (63, 63, 1024, 1024, 1, 0.0),
    (100, 37, 130, 136, 0, 1.0), (255, 255, 512, 512, 1, 1.0), (128, 256, 64, 64, 0, 0.0),
    (129, 129, 200, 200, 1, 0.0),
    # m > 256: two row halves of A, each a work item over the same X tile
    (511, 511, 4096, 4096, 1, 0.0), (511, 511, 1024, 1024, 0, 1.0), (300, 400, 200, 200, 1, 0.0),
    (257, 129, 130, 136, 0, 1.0), (511, 300, 512, 512, 1, 1.0), (200, 511, 256, 256, 0, 0.0)])
def test_bf16x3_gemm(cuda, m, k, ncols, ldx, cplx_, beta):
    rng = np.random.default_rng(m * 7 + ncols)
    A = rng.normal(size=(m, k))
    X = rng.normal(size=(k, ldx)).astype(np.float32)
    Y0 = rng.normal(size=(m, ncols)).astype(np.float32)
    al = (0.5 - 1.25j) if cplx_ else 0.75
    T = A @ X[:, :ncols].astype(np.float64)
    if cplx_:
        Tc = T[:, 0::2] + 1j * T[:, 1::2]
        Rc = beta * (Y0[:, 0::2] + 1j * Y0[:, 1::2]) + al * Tc
        ref = np.empty((m, ncols))
        ref[:, 0::2], ref[:, 1::2] = Rc.real, Rc.imag
    else:
        ref = beta * Y0 + al * T
    Ap = prepare(A)
    Xd = torch.from_numpy(X).cuda()
    Yd = torch.from_numpy(Y0.copy()).cuda()
    a = complex(al)
    _lib.load().ccl_dht_bf16x3_status(1)
    call("ccl_dht_bf16x3_gemm_batch", 1, m, k, ints([ncols]), cplx_, PP([Ap]), PP([Xd]),
         longs([ldx]), PP([Yd]), longs([ncols]), a.real, a.imag, beta, _lib.stream())
    torch.cuda.synchronize()
    assert _lib.load().ccl_dht_bf16x3_status(1) == 0
    err = np.abs(Yd.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < TOL, err


def test_bf16x3_batch_mixed_entries(cuda):
    """Real (m=0) and complex-as-real (m>=1) entries with different column
    counts and matrices in one launch."""
    rng = np.random.default_rng(3)
    m = k = 255
    mats = [rng.normal(size=(m, k)), rng.normal(size=(m, k))]
    preps = [prepare(a, CCL_F32) for a in mats]
    ncols = [2048, 4096, 2048]
    which = [0, 1, 0]
    Xs = [rng.normal(size=(k, n)).astype(np.float32) for n in ncols]
    Xd = [torch.from_numpy(x).cuda() for x in Xs]
    Yd = [torch.empty((m, n), dtype=torch.float32, device="cuda") for n in ncols]
    call("ccl_dht_bf16x3_gemm_batch", 3, m, k, ints(ncols), 0, PP([preps[w] for w in which]),
         PP(Xd), longs(ncols), PP(Yd), longs(ncols), 1.0, 0.0, 0.0, _lib.stream())
    torch.cuda.synchronize()
    assert _lib.load().ccl_dht_bf16x3_status(1) == 0
    for i in range(3):
        ref = mats[which[i]].astype(np.float32).astype(np.float64) @ Xs[i].astype(np.float64)
        err = np.abs(Yd[i].cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err < TOL, (i, err)


def test_bf16x3_rejects_large_k_and_misaligned(cuda):
    import ctypes
    lib = _lib.load()
    nb = ctypes.c_size_t(0)
    assert lib.ccl_dht_bf16x3_prepare_bytes(511, 511, ctypes.byref(nb)) == 0
    assert nb.value == 2 * 16 * 2 * 256 * 32 * 2  # two halves of 16 chunks, hi + lo
    assert lib.ccl_dht_bf16x3_prepare_bytes(513, 64, ctypes.byref(nb)) == 3
    assert lib.ccl_dht_bf16x3_prepare_bytes(64, 513, ctypes.byref(nb)) == 3
    t = torch.zeros(1 << 20, dtype=torch.float32, device="cuda")
    p = t.data_ptr()
    rc = lib.ccl_dht_bf16x3_gemm_batch(1, 64, 64, ints([64]), 0, PP([p]), PP([p + 4]),
                                       longs([64]), PP([p]), longs([64]), 1.0, 0.0, 0.0, None)
    assert rc == 1 and b"aligned" in lib.ccl_last_error()


def test_bf16x3_batch_many_items(cuda):
    """More work items than CTAs: each CTA walks several N tiles and reloads
    its resident A tile when the (entry, M tile) changes; complex alpha and
    accumulation into Y."""
    rng = np.random.default_rng(11)
    m = k = 255
    mats = [rng.normal(size=(m, k)) for _ in range(3)]
    preps = [prepare(a, CCL_F32) for a in mats]
    ncols = [4096, 2048, 4096, 4096, 1000, 4096, 2048, 4096]
    which = [0, 1, 2, 0, 1, 2, 0, 1]
    al = 0.5 - 1.25j
    Xs = [rng.normal(size=(k, n)).astype(np.float32) for n in ncols]
    Y0 = [rng.normal(size=(m, n)).astype(np.float32) for n in ncols]
    Xd = [torch.from_numpy(x).cuda() for x in Xs]
    Yd = [torch.from_numpy(y.copy()).cuda() for y in Y0]
    call("ccl_dht_bf16x3_gemm_batch", len(ncols), m, k, ints(ncols), 1,
         PP([preps[w] for w in which]), PP(Xd), longs(ncols), PP(Yd), longs(ncols),
         al.real, al.imag, 1.0, _lib.stream())
    torch.cuda.synchronize()
    assert _lib.load().ccl_dht_bf16x3_status(1) == 0
    for i in range(len(ncols)):
        A32 = mats[which[i]].astype(np.float32).astype(np.float64)
        T = A32 @ Xs[i].astype(np.float64)
        Rc = (Y0[i][:, 0::2] + 1j * Y0[i][:, 1::2]) + al * (T[:, 0::2] + 1j * T[:, 1::2])
        ref = np.empty_like(T)
        ref[:, 0::2], ref[:, 1::2] = Rc.real, Rc.imag
        err = np.abs(Yd[i].cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err < TOL, (i, err)


def test_bf16x3_batch_large_modes(cuda):
    """The 4096 x 512 grid's transforms: m = k = 511, a batch of complex
    and real entries with different matrices, accumulation into Y."""
    rng = np.random.default_rng(17)
    m = k = 511
    mats = [rng.normal(size=(m, k)) for _ in range(2)]
    preps = [prepare(a, CCL_F32) for a in mats]
    ncols = [8192, 4096, 8192, 1000]
    which = [0, 1, 1, 0]
    Xs = [rng.normal(size=(k, n)).astype(np.float32) for n in ncols]
    Y0 = [rng.normal(size=(m, n)).astype(np.float32) for n in ncols]
    Xd = [torch.from_numpy(x).cuda() for x in Xs]
    Yd = [torch.from_numpy(y.copy()).cuda() for y in Y0]
    call("ccl_dht_bf16x3_gemm_batch", len(ncols), m, k, ints(ncols), 0,
         PP([preps[w] for w in which]), PP(Xd), longs(ncols), PP(Yd), longs(ncols),
         -0.5, 0.0, 1.0, _lib.stream())
    torch.cuda.synchronize()
    assert _lib.load().ccl_dht_bf16x3_status(1) == 0
    for i in range(len(ncols)):
        A32 = mats[which[i]].astype(np.float32).astype(np.float64)
        ref = Y0[i] - 0.5 * (A32 @ Xs[i].astype(np.float64))
        err = np.abs(Yd[i].cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err < TOL, (i, err)


def test_bf16x3_repeated_launches(cuda):
    """Back-to-back launches over many work items must each give the same,
    correct result (a stage-ring reuse race shows up only intermittently)."""
    rng = np.random.default_rng(5)
    m = k = 255
    A = rng.normal(size=(m, k))
    Ap = prepare(A, CCL_F32)
    b, n = 6, 4096
    Xs = [rng.normal(size=(k, n)).astype(np.float32) for _ in range(b)]
    Xd = [torch.from_numpy(x).cuda() for x in Xs]
    Yd = [torch.empty((m, n), dtype=torch.float32, device="cuda") for _ in range(b)]
    A32 = A.astype(np.float32).astype(np.float64)
    refs = [A32 @ x.astype(np.float64) for x in Xs]
    first = None
    for it in range(8):
        for y in Yd:
            y.fill_(float("nan"))
        call("ccl_dht_bf16x3_gemm_batch", b, m, k, ints([n] * b), 0, PP([Ap] * b), PP(Xd),
             longs([n] * b), PP(Yd), longs([n] * b), 1.0, 0.0, 0.0, _lib.stream())
        torch.cuda.synchronize()
        assert _lib.load().ccl_dht_bf16x3_status(1) == 0
        got = [y.cpu().numpy() for y in Yd]
        for i in range(b):
            err = np.abs(got[i] - refs[i]).max() / np.abs(refs[i]).max()
            assert err < TOL, (it, i, err)
        if first is None:
            first = got
        else:
            for i in range(b):
                assert np.array_equal(first[i], got[i]), (it, i)
