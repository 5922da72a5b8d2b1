"""Kernel-level parity of the CUDA library against the oracle, through the
C ABI.  Integer outputs (keys, counts, offsets, sort order) must be
identical; the FP64 particle, grid and elementwise kernels reproduce the
reference's arithmetic term by term (compiled without FMA contraction), so
they are compared bit for bit as well; the FFT and the Hankel GEMM use other
summation orders than numpy and are held to 1e-13 of the array's largest
magnitude."""
import ctypes as C

import numpy as np
import pytest
import torch

from chimeracl_gb300 import _lib
from chimeracl_gb300._lib import CCL_F32, CCL_F64, PP, call

pytestmark = pytest.mark.gpu

FFT_TOL = 1e-13


def geom(Nx=96, Nr=24, Xmin=-10.0, Xmax=0.0, Rmax=5.0):
    dx = (Xmax - Xmin) / (Nx - 1)
    dr = Rmax / (Nr - 1.5)
    return dict(Nx=Nx, Nr=Nr, Xmin=Xmin, Xmax=Xmax, Rmax=Rmax, dx=dx, dr=dr, dx_inv=1.0 / dx,
                Rmin=-0.5 * dr, dr_inv=1.0 / dr)


def particles(rng, n, g, spill=0.15, boundaries=True):
    L = g["Xmax"] - g["Xmin"]
    x = rng.uniform(g["Xmin"] - spill * L, g["Xmax"] + spill * L, n)
    r = rng.uniform(0, g["Rmax"] * (1 + spill), n)
    if boundaries:  # particles exactly on cell faces
        k = n // 8
        x[:k] = g["Xmin"] + g["dx"] * rng.integers(0, g["Nx"], k)
        r[k:2 * k] = g["Rmin"] + g["dr"] * rng.integers(1, g["Nr"], k)
    th = rng.uniform(0, 2 * np.pi, n)
    y, z = r * np.cos(th), r * np.sin(th)
    u = rng.normal(0, 0.7, (3, n))
    g_inv = 1.0 / np.sqrt(1 + (u ** 2).sum(0))
    w = rng.uniform(0.5, 1.5, n) * r
    return dict(x=x, y=y, z=z, px=u[0].copy(), py=u[1].copy(), pz=u[2].copy(), g_inv=g_inv, w=w)


# Uploads stay referenced until the test ends: a tensor created inline in a
# call's argument list would otherwise be freed, and its memory handed to the
# next upload, before the kernel that reads it is enqueued.
_KEEP = []


@pytest.fixture(autouse=True)
def _keep_alive():
    yield
    torch.cuda.synchronize()
    _KEEP.clear()


def dev(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    t = torch.from_numpy(a.copy()).cuda()
    _KEEP.append(t)
    return t


def host(t, dtype=None):
    a = t.cpu().numpy()
    if dtype == np.uint32:
        a = a.view(np.uint32)
    return a


def S():
    return _lib.stream()


def oracle_sort(port, p, g):
    n = p["x"].size
    C_ = (g["Nx"] - 1) * (g["Nr"] - 1)
    indx = np.empty(n, np.uint32)
    cnt = np.zeros(C_ + 1, np.uint32)
    port.index_and_sum(p["x"], p["y"], p["z"], cnt, indx, g["Nx"], g["Xmin"], g["dx_inv"],
                       g["Nr"], g["Rmin"], g["dr_inv"])
    off = np.zeros(C_ + 2, np.uint32)
    off[1:] = np.cumsum(cnt.astype(np.int64)).astype(np.uint32)
    srt = np.empty(n, np.uint32)
    port.sort(off, indx, np.zeros_like(cnt), srt)
    return indx, cnt, off, srt


def gpu_sort(p, g):
    n = p["x"].size
    C_ = (g["Nx"] - 1) * (g["Nr"] - 1)
    x, y, z = dev(p["x"]), dev(p["y"]), dev(p["z"])
    i32 = dict(dtype=torch.int32, device="cuda")
    indx, cnt = torch.empty(max(n, 1), **i32), torch.empty(C_ + 1, **i32)
    off, srt, nst = torch.empty(C_ + 2, **i32), torch.empty(max(n, 1), **i32), torch.empty(1, **i32)
    wsb = _lib.sort_workspace_bytes(n, C_)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    call("ccl_index_sort", CCL_F64, n, x.data_ptr(), y.data_ptr(), z.data_ptr(), g["Nx"],
         g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"], indx.data_ptr(), cnt.data_ptr(),
         off.data_ptr(), srt.data_ptr(), nst.data_ptr(), ws.data_ptr(), wsb, S())
    torch.cuda.synchronize()
    return (host(indx, np.uint32)[:n], host(cnt, np.uint32), host(off, np.uint32),
            host(srt, np.uint32)[:n], int(host(nst)[0]))


# ----------------------------------------------------------------------- sort
@pytest.mark.parametrize("n,Nx,Nr", [(0, 32, 8), (1, 32, 8), (5000, 96, 24), (300000, 512, 64),
                                     (200000, 2048, 256)])
def test_index_sort_bit_exact(cuda, port, n, Nx, Nr):
    rng = np.random.default_rng(n + Nx)
    g = geom(Nx, Nr)
    p = particles(rng, n, g)
    oi, oc, oo, osr = oracle_sort(port, p, g)
    gi, gc, go, gsr, nst = gpu_sort(p, g)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gc, oc)
    np.testing.assert_array_equal(go, oo)
    np.testing.assert_array_equal(gsr, osr)  # stable: ascending index within each cell
    assert nst == int(oo[-2])


def test_index_sort_presorted_and_clustered(cuda, port):
    # cell-ordered input (after an align) and a dense cluster in few cells
    rng = np.random.default_rng(7)
    g = geom(256, 32)
    p = particles(rng, 100000, g, spill=0.0, boundaries=False)
    _, _, _, srt = oracle_sort(port, p, g)
    p = {k: v[srt].copy() for k, v in p.items()}
    p["x"][:20000] = g["Xmin"] + 10.3 * g["dx"]
    p["y"][:20000] = 1.1 * g["dr"]
    p["z"][:20000] = 0.0
    for a, b in zip(oracle_sort(port, p, g), gpu_sort(p, g)[:4]):
        np.testing.assert_array_equal(b, a)


def test_index_sort_nearly_sorted_full_size(cuda, port):
    # the step's case: cell-ordered particles moved by less than a cell,
    # 2048 x 256 nodes at about 8 per cell
    rng = np.random.default_rng(8)
    g = geom(2048, 256)
    p = particles(rng, 4_000_000, g, spill=0.0, boundaries=False)
    _, _, _, srt = oracle_sort(port, p, g)
    p = {k: v[srt].copy() for k, v in p.items()}
    p["x"] += rng.uniform(-0.4, 0.4, p["x"].size) * g["dx"]
    p["y"] += rng.uniform(-0.4, 0.4, p["y"].size) * g["dr"]
    for a, b in zip(oracle_sort(port, p, g), gpu_sort(p, g)[:4]):
        np.testing.assert_array_equal(b, a)
    assert _lib.load().ccl_sort_status(1) == 0  # no bounded wait of the scan gave up


def test_index_sort_many_scan_tiles(cuda, port):
    # 4096 x 512 nodes: 2.09M cells, about a thousand tiles of the offsets'
    # single-pass scan; random particle order (most cells claimed by many
    # warps), then the same workspace again on a cell-ordered copy
    rng = np.random.default_rng(9)
    g = geom(4096, 512)
    p = particles(rng, 2_000_000, g)
    o = oracle_sort(port, p, g)
    for a, b in zip(o, gpu_sort(p, g)[:4]):
        np.testing.assert_array_equal(b, a)
    q = {k: v[o[3]].copy() for k, v in p.items()}
    for a, b in zip(oracle_sort(port, q, g), gpu_sort(q, g)[:4]):
        np.testing.assert_array_equal(b, a)
    assert _lib.load().ccl_sort_status(1) == 0


def test_index_sort_workspace_too_small(cuda):
    g = geom()
    n = 100
    C_ = (g["Nx"] - 1) * (g["Nr"] - 1)
    t = torch.zeros(4 * (n + C_ + 8), dtype=torch.int32, device="cuda")
    lib = _lib.load()
    rc = lib.ccl_index_sort(CCL_F64, n, t.data_ptr(), t.data_ptr(), t.data_ptr(), g["Nx"],
                            g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"], t.data_ptr(),
                            t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(),
                            16, S())
    assert rc == 4 and b"workspace" in lib.ccl_last_error()


# ------------------------------------------------------------------ particles
def test_push_x_bit_exact(cuda, port):
    rng = np.random.default_rng(1)
    p = particles(rng, 100001, geom())
    d = {k: dev(v) for k, v in p.items()}
    call("ccl_push_x", CCL_F64, p["x"].size, d["x"].data_ptr(), d["y"].data_ptr(),
         d["z"].data_ptr(), d["px"].data_ptr(), d["py"].data_ptr(), d["pz"].data_ptr(),
         d["g_inv"].data_ptr(), 0.0217, S())
    port.push_xyz(p["x"], p["y"], p["z"], p["px"], p["py"], p["pz"], p["g_inv"], 0.0217)
    for k in ("x", "y", "z"):
        np.testing.assert_array_equal(host(d[k]), p[k])


def compensated_push_np(hi, lo, p, g_inv, dt):
    """numpy restatement of ccl_push_x_compensated for one coordinate, in
    the arrays' own type (IEEE round-to-nearest, like the kernel's _rn adds):
    d as push_xyz forms it, Knuth's two-sum of hi + d, the error added to
    lo, Dekker's fast two-sum renormalisation."""
    t = hi.dtype.type
    d = p * (t(dt) * g_inv)
    s = hi + d
    bp = s - hi
    e = (hi - (s - bp)) + (d - bp)
    l = lo + e
    h2 = s + l
    return h2, l - (h2 - s)


@pytest.mark.parametrize("dtype", [CCL_F32, CCL_F64])
def test_push_x_compensated_bit_exact(cuda, dtype):
    rng = np.random.default_rng(11)
    npt = np.float32 if dtype == CCL_F32 else np.float64
    p = {k: v.astype(npt) for k, v in particles(rng, 100003, geom(Xmin=-90.0, Xmax=-10.0)).items()}
    for k in ("x", "y", "z"):  # some low parts already carried
        p[k + "_lo"] = (rng.uniform(-0.5, 0.5, p[k].size) * np.spacing(p[k])).astype(npt)
    names = ("x", "y", "z", "x_lo", "y_lo", "z_lo", "px", "py", "pz", "g_inv")
    d = {k: dev(p[k]) for k in names}
    for _ in range(3):
        call("ccl_push_x_compensated", dtype, p["x"].size, *[d[k].data_ptr() for k in names],
             0.0195, S())
        for c in ("x", "y", "z"):
            p[c], p[c + "_lo"] = compensated_push_np(p[c], p[c + "_lo"], p["p" + c], p["g_inv"],
                                                     0.0195)
    for k in ("x", "y", "z", "x_lo", "y_lo", "z_lo"):
        np.testing.assert_array_equal(host(d[k]), p[k], err_msg=k)
    # the renormalised pair: hi is the nearest value to hi + lo
    for c in ("x", "y", "z"):
        assert np.all(np.abs(p[c + "_lo"]) <= 0.5 * np.spacing(np.abs(p[c])))


def test_push_x_compensated_tracks_exact_sum(cuda):
    """1000 pushes of slow and fast particles at |x| ~ 60: the compensated
    FP32 coordinate hi + lo stays within 1e-2 FP32 units in the last place of
    the exact sum of its FP32 displacements, where the plain FP32 push loses
    up to half a unit per push (and a displacement below that is lost
    whole: a slow particle does not move)."""
    rng = np.random.default_rng(12)
    n, steps, dt = 65536, 1000, 0.0195
    x = rng.uniform(-70.0, -50.0, n)
    y, z = rng.uniform(-30.0, 30.0, (2, n))
    u = rng.normal(0, 1.0, (3, n)) * np.repeat([1e-5, 1e-3, 1e-1, 1.0], n // 4)
    g_inv = 1.0 / np.sqrt(1 + (u ** 2).sum(0))
    f32 = {k: v.astype(np.float32) for k, v in dict(x=x, y=y, z=z, px=u[0], py=u[1], pz=u[2],
                                                      g_inv=g_inv).items()}
    comp = {k: dev(v) for k, v in f32.items()}
    plain = {k: dev(v) for k, v in f32.items()}
    for c in ("x", "y", "z"):
        comp[c + "_lo"] = dev(np.zeros(n, np.float32))
    cn = ("x", "y", "z", "x_lo", "y_lo", "z_lo", "px", "py", "pz", "g_inv")
    pn = ("x", "y", "z", "px", "py", "pz", "g_inv")
    for _ in range(steps):
        call("ccl_push_x_compensated", CCL_F32, n, *[comp[k].data_ptr() for k in cn], dt, S())
        call("ccl_push_x", CCL_F32, n, *[plain[k].data_ptr() for k in pn], dt, S())
    dt_g = np.float32(dt) * f32["g_inv"]
    for c in ("x", "y", "z"):
        d = (f32["p" + c] * dt_g).astype(np.float64)  # the kernel's displacement
        exact = f32[c].astype(np.float64) + steps * d
        ulp = np.spacing(np.maximum(np.abs(exact), np.abs(f32[c])).astype(np.float32))
        ec = np.abs(host(comp[c]).astype(np.float64) + host(comp[c + "_lo"]) - exact) / ulp
        ep = np.abs(host(plain[c]).astype(np.float64) - exact) / ulp
        assert ec.max() < 1e-2, (c, ec.max())
        assert ep.max() > 10.0, (c, ep.max())


def test_align_bit_exact(cuda, port):
    rng = np.random.default_rng(2)
    g = geom()
    p = particles(rng, 20000, g)
    _, _, off, srt = oracle_sort(port, p, g)
    ns = int(off[-2])
    names = list(p)
    src = [dev(p[k]) for k in names]
    dst = [torch.empty(ns, dtype=torch.float64, device="cuda") for _ in names]
    call("ccl_align", CCL_F64, ns, len(names), PP(src), PP(dst), dev(srt).data_ptr(), S())
    for k, t in zip(names, dst):
        ref = np.empty(ns)
        port.data_align(p[k], ref, srt)
        np.testing.assert_array_equal(host(t), ref)


def test_fill_grid_and_profile(cuda, port):
    rng = np.random.default_rng(3)
    Nx_loc, Nr_loc = 21, 17
    xg = -3.0 + 0.05 * np.arange(Nx_loc)
    rg = 0.0 + 0.3 * np.arange(Nr_loc)
    nc = (Nx_loc - 1) * (Nr_loc - 1)
    theta = rng.uniform(0, 2 * np.pi, nc)
    npp = (2, 2, 4)
    n = nc * 16
    out = [np.empty(n) for _ in range(4)]
    port.fill_grid(*out, theta, xg, rg, Nx_loc, *npp)
    d = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(4)]
    call("ccl_fill_grid", CCL_F64, nc, *[t.data_ptr() for t in d], dev(theta).data_ptr(),
         dev(xg).data_ptr(), dev(rg).data_ptr(), Nx_loc, *npp, S())
    np.testing.assert_array_equal(host(d[0]), out[0])  # x: no transcendental
    np.testing.assert_array_equal(host(d[3]), out[3])  # w = r
    for k in (1, 2):  # y, z = r sin/cos: CUDA vs libm sin/cos, a few ulp
        np.testing.assert_allclose(host(d[k]), out[k], rtol=0, atol=4e-16 * rg.max())
    # density profile on the filled x
    xk = np.array([-10.0, -2.6, -2.1, 5.0])
    fk = np.array([0.0, 0.0, 1.0, 1.0])
    dxm1 = 1.0 / (xk[1:] - xk[:-1])
    w_ref = out[3].copy()
    port.profile_by_interpolant(out[0], w_ref, xk, fk, dxm1)
    call("ccl_dens_profile", CCL_F64, n, d[0].data_ptr(), d[3].data_ptr(), dev(xk).data_ptr(),
         dev(fk).data_ptr(), dev(dxm1).data_ptr(), xk.size, S())
    np.testing.assert_array_equal(host(d[3]), w_ref)


# ----------------------------------------------------------------------- grid
def fields(rng, Nr, Nx, M, names):
    out = {}
    for n in names:
        out[n + "_m0"] = rng.normal(size=(Nr, Nx))
        for m in range(1, M + 1):
            out[n + "_m" + str(m)] = rng.normal(size=(Nr, Nx)) + 1j * rng.normal(size=(Nr, Nx))
    return out


@pytest.mark.parametrize("M", [0, 1, 2])
@pytest.mark.parametrize("vec", [False, True])
def test_deposit_bit_exact(cuda, port, M, vec):
    rng = np.random.default_rng(10 + M + 5 * vec)
    g = geom(160, 40)
    p = particles(rng, 60000, g)
    _, _, off, srt = oracle_sort(port, p, g)
    names = ["J" + c for c in "xyz"] if vec else ["rho"]
    f0 = fields(rng, g["Nr"], g["Nx"], M, names)  # deposits add to existing values
    ref = {k: v.copy() for k, v in f0.items()}
    order = [n + "_m" + str(m) for m in range(M + 1) for n in names]
    nxnr4 = (g["Nr"]) // 2 * (g["Nx"]) // 2
    charge = -1
    if vec:
        port.depose_vector(M, nxnr4, srt, p["x"], p["y"], p["z"], p["px"], p["py"], p["pz"],
                           p["g_inv"], p["w"], off, charge, g["Nx"], g["Xmin"], g["dx_inv"],
                           g["Nr"], g["Rmin"], g["dr_inv"], [ref[k] for k in order])
    else:
        port.depose_scalar(M, nxnr4, srt, p["x"], p["y"], p["z"], p["w"], off, charge, g["Nx"],
                           g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"],
                           [ref[k] for k in order])
    d = {k: dev(v) for k, v in f0.items()}
    pd = {k: dev(v) for k, v in p.items()}
    args = (g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"])
    if vec:
        call("ccl_deposit_vector", CCL_F64, M, dev(srt).data_ptr(), dev(off).data_ptr(),
             pd["x"].data_ptr(), pd["y"].data_ptr(), pd["z"].data_ptr(), pd["px"].data_ptr(),
             pd["py"].data_ptr(), pd["pz"].data_ptr(), pd["g_inv"].data_ptr(), pd["w"].data_ptr(),
             charge, *args, PP([d[k] for k in order]), S())
    else:
        call("ccl_deposit_scalar", CCL_F64, M, dev(srt).data_ptr(), dev(off).data_ptr(),
             pd["x"].data_ptr(), pd["y"].data_ptr(), pd["z"].data_ptr(), pd["w"].data_ptr(),
             charge, *args, PP([d[k] for k in order]), S())
    for k in order:
        np.testing.assert_array_equal(host(d[k]), ref[k], err_msg=k)


def to32(a):
    return a.astype(np.complex64 if np.iscomplexobj(a) else np.float32)


def to64(a):
    return a.astype(np.complex128 if np.iscomplexobj(a) else np.float64)


@pytest.mark.parametrize("M,vec", [(0, False), (1, False), (1, True), (2, True)])
def test_deposit_fp32(cuda, port, M, vec):
    """The FP32 deposit (row-staged kernel) against the FP64 oracle on the
    same FP32 inputs, with one dense cluster so that a tile row holds more
    particles than one staging round (relative 1e-5 of the deposited
    magnitude: FP32 sums of a few hundred terms)."""
    rng = np.random.default_rng(40 + M + 5 * vec)
    g = geom(160, 40)
    p = particles(rng, 60000, g)
    p["x"][:3000] = g["Xmin"] + g["dx"] * rng.uniform(20.1, 27.9, 3000)
    p["y"][:3000] = g["dr"] * rng.uniform(5.1, 5.9, 3000)
    p["z"][:3000] = 0.0
    p = {k: v.astype(np.float32).astype(np.float64) for k, v in p.items()}
    _, _, off, srt = oracle_sort(port, p, g)
    names = ["J" + c for c in "xyz"] if vec else ["rho"]
    f0 = {k: to64(to32(v)) for k, v in fields(rng, g["Nr"], g["Nx"], M, names).items()}
    ref = {k: v.copy() for k, v in f0.items()}
    order = [n + "_m" + str(m) for m in range(M + 1) for n in names]
    nxnr4 = (g["Nr"]) // 2 * (g["Nx"]) // 2
    charge = -1
    if vec:
        port.depose_vector(M, nxnr4, srt, p["x"], p["y"], p["z"], p["px"], p["py"], p["pz"],
                           p["g_inv"], p["w"], off, charge, g["Nx"], g["Xmin"], g["dx_inv"],
                           g["Nr"], g["Rmin"], g["dr_inv"], [ref[k] for k in order])
    else:
        port.depose_scalar(M, nxnr4, srt, p["x"], p["y"], p["z"], p["w"], off, charge, g["Nx"],
                           g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"],
                           [ref[k] for k in order])
    d = {k: dev(to32(v)) for k, v in f0.items()}
    pd = {k: dev(to32(v)) for k, v in p.items()}
    args = (g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"])
    if vec:
        call("ccl_deposit_vector", CCL_F32, M, dev(srt).data_ptr(), dev(off).data_ptr(),
             pd["x"].data_ptr(), pd["y"].data_ptr(), pd["z"].data_ptr(), pd["px"].data_ptr(),
             pd["py"].data_ptr(), pd["pz"].data_ptr(), pd["g_inv"].data_ptr(), pd["w"].data_ptr(),
             charge, *args, PP([d[k] for k in order]), S())
    else:
        call("ccl_deposit_scalar", CCL_F32, M, dev(srt).data_ptr(), dev(off).data_ptr(),
             pd["x"].data_ptr(), pd["y"].data_ptr(), pd["z"].data_ptr(), pd["w"].data_ptr(),
             charge, *args, PP([d[k] for k in order]), S())
    for k in order:
        inc = ref[k] - f0[k]
        got = host(d[k])
        assert got.shape == ref[k].shape and got.dtype == to32(ref[k]).dtype
        err = np.abs(to64(got) - ref[k]).max() / np.abs(inc).max()
        assert err < 1e-5, (k, err)


@pytest.mark.parametrize("M", [0, 1, 2])
def test_postproc_and_warp_axis_bit_exact(cuda, port, M):
    rng = np.random.default_rng(20 + M)
    g = geom(64, 16)
    names = ["Jx", "Jy", "Jz"]
    f0 = fields(rng, g["Nr"], g["Nx"], M, names)
    dv = np.where(np.arange(g["Nr"]) > 0, rng.uniform(0.1, 2.0, g["Nr"]), 0.0)
    order = [n + "_m" + str(m) for n in names for m in range(M + 1)]
    ref = {k: v.copy() for k, v in f0.items()}
    for k in order:
        port.treat_axis(ref[k], g["Nx"])
        port.divide_by_dv(ref[k], g["Nx"], dv)
    d = {k: dev(v) for k, v in f0.items()}
    call("ccl_deposit_postproc", CCL_F64, M, 3, PP([d[k] for k in order]), g["Nx"], g["Nr"],
         dev(dv).data_ptr(), S())
    for k in order:
        np.testing.assert_array_equal(host(d[k]), ref[k], err_msg=k)
    for k in order:
        port.warp_axis(ref[k], g["Nx"], int(k[-1]))
    call("ccl_warp_axis", CCL_F64, M, 3, PP([d[k] for k in order]), g["Nx"], S())
    for k in order:
        np.testing.assert_array_equal(host(d[k]), ref[k], err_msg=k)


@pytest.mark.parametrize("M", [0, 1, 2])
def test_gather_push_bit_exact(cuda, port, M):
    rng = np.random.default_rng(30 + M)
    g = geom(128, 32)
    p = particles(rng, 50000, g)
    _, _, off, srt = oracle_sort(port, p, g)
    np_stay = int(off[-2])
    names = ["E" + c for c in "xyz"] + ["B" + c for c in "xyz"]
    f = fields(rng, g["Nr"], g["Nx"], M, names)
    order = [n + "_m" + str(m) for m in range(M + 1) for n in names]
    ref = {k: p[k].copy() for k in ("px", "py", "pz", "g_inv")}
    fp = 0.37
    port.gather_and_push(M, p["x"], p["y"], p["z"], ref["px"], ref["py"], ref["pz"], ref["g_inv"],
                         srt, fp, p["x"].size, np_stay, g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"],
                         g["Rmin"], g["dr_inv"], [f[k] for k in order])
    pd = {k: dev(v) for k, v in p.items()}
    fd = [dev(f[k]) for k in order]
    nst = torch.tensor([np_stay], dtype=torch.int32, device="cuda")
    call("ccl_gather_push", CCL_F64, M, p["x"].size, pd["x"].data_ptr(), pd["y"].data_ptr(),
         pd["z"].data_ptr(), pd["px"].data_ptr(), pd["py"].data_ptr(), pd["pz"].data_ptr(),
         pd["g_inv"].data_ptr(), dev(srt).data_ptr(), nst.data_ptr(), fp, g["Nx"], g["Xmin"],
         g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"], PP(fd), S())
    for k in ref:
        np.testing.assert_array_equal(host(pd[k]), ref[k], err_msg=k)


@pytest.mark.parametrize("cells", [False, True])
@pytest.mark.parametrize("M", [0, 1, 2, 3])
def test_gather_push_fp32(cuda, port, M, cells):
    """The FP32 gather + Boris kernel against the FP64 oracle on the same
    FP32-rounded inputs (no particles exactly on cell faces, where the two
    precisions may pick different but equivalent cells); `cells` runs the
    tiled form (ccl_gather_push_cells)."""
    rng = np.random.default_rng(50 + M)
    g = geom(128, 32)
    p = {k: to64(to32(v)) for k, v in particles(rng, 50000, g, boundaries=False).items()}
    _, _, off, srt = oracle_sort(port, p, g)
    np_stay = int(off[-2])
    names = ["E" + c for c in "xyz"] + ["B" + c for c in "xyz"]
    f = {k: to64(to32(v)) for k, v in fields(rng, g["Nr"], g["Nx"], M, names).items()}
    order = [n + "_m" + str(m) for m in range(M + 1) for n in names]
    ref = {k: p[k].copy() for k in ("px", "py", "pz", "g_inv")}
    fp = 0.37
    port.gather_and_push(M, p["x"], p["y"], p["z"], ref["px"], ref["py"], ref["pz"], ref["g_inv"],
                         srt, fp, p["x"].size, np_stay, g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"],
                         g["Rmin"], g["dr_inv"], [f[k] for k in order])
    pd = {k: dev(to32(v)) for k, v in p.items()}
    fd = [dev(to32(f[k])) for k in order]
    nst = torch.tensor([np_stay], dtype=torch.int32, device="cuda")
    if cells:
        call("ccl_gather_push_cells", CCL_F32, M, p["x"].size, pd["x"].data_ptr(),
             pd["y"].data_ptr(), pd["z"].data_ptr(), pd["px"].data_ptr(), pd["py"].data_ptr(),
             pd["pz"].data_ptr(), pd["g_inv"].data_ptr(), dev(srt).data_ptr(),
             dev(off).data_ptr(), nst.data_ptr(), fp, g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"],
             g["Rmin"], g["dr_inv"], PP(fd), S())
    else:
        call("ccl_gather_push", CCL_F32, M, p["x"].size, pd["x"].data_ptr(), pd["y"].data_ptr(),
             pd["z"].data_ptr(), pd["px"].data_ptr(), pd["py"].data_ptr(), pd["pz"].data_ptr(),
             pd["g_inv"].data_ptr(), dev(srt).data_ptr(), nst.data_ptr(), fp, g["Nx"],
             g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"], PP(fd), S())
    for k in ref:
        got = to64(host(pd[k]))
        err = np.abs(got - ref[k]).max() / np.abs(ref[k]).max()
        assert err < 2e-5, (k, err)


def _split(p):
    """Coordinates as FP32 value + FP32 residual; the other components
    rounded to FP32 (only coordinates carry low parts)."""
    q = {k: to32(v) for k, v in p.items()}
    lo = {k: to32(p[k] - to64(q[k])) for k in ("x", "y", "z")}
    ref = {k: to64(q[k]) for k in p}
    for k in ("x", "y", "z"):
        ref[k] = p[k]  # the oracle takes the double coordinates
    return q, lo, ref


@pytest.mark.parametrize("M,vec", [(0, False), (1, False), (1, True)])
def test_deposit_fp32_low_parts(cuda, port, M, vec):
    """Compensated FP32 coordinates (hi + lo) at x ~ -1e4, where the FP32
    spacing is 8e-3 of a cell: the _lo deposit against the FP64 oracle on the
    double coordinates within 2e-5 of the deposited magnitude, the same
    deposit from hi alone at least 10x further off."""
    rng = np.random.default_rng(60 + M + 5 * vec)
    g = geom(160, 40, Xmin=-10020.0, Xmax=-10000.0)
    q, lo, p = _split(particles(rng, 60000, g, boundaries=False))
    _, _, off, srt = oracle_sort(port, p, g)
    names = ["J" + c for c in "xyz"] if vec else ["rho"]
    f0 = {k: to64(to32(v)) for k, v in fields(rng, g["Nr"], g["Nx"], M, names).items()}
    ref = {k: v.copy() for k, v in f0.items()}
    order = [n + "_m" + str(m) for m in range(M + 1) for n in names]
    nxnr4 = (g["Nr"]) // 2 * (g["Nx"]) // 2
    geo = (g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"])
    if vec:
        port.depose_vector(M, nxnr4, srt, p["x"], p["y"], p["z"], p["px"], p["py"], p["pz"],
                           p["g_inv"], p["w"], off, -1, *geo, [ref[k] for k in order])
    else:
        port.depose_scalar(M, nxnr4, srt, p["x"], p["y"], p["z"], p["w"], off, -1, *geo,
                           [ref[k] for k in order])
    pd = {k: dev(v) for k, v in q.items()}
    ld = [dev(lo[k]).data_ptr() for k in ("x", "y", "z")]
    errs = []
    for use_lo in (True, False):
        d = {k: dev(to32(v)) for k, v in f0.items()}
        if vec:
            args = [CCL_F32, M, dev(srt).data_ptr(), dev(off).data_ptr(), pd["x"].data_ptr(),
                    pd["y"].data_ptr(), pd["z"].data_ptr(), pd["px"].data_ptr(),
                    pd["py"].data_ptr(), pd["pz"].data_ptr(), pd["g_inv"].data_ptr(),
                    pd["w"].data_ptr(), -1, *geo, PP([d[k] for k in order])]
            name = "ccl_deposit_vector"
        else:
            args = [CCL_F32, M, dev(srt).data_ptr(), dev(off).data_ptr(), pd["x"].data_ptr(),
                    pd["y"].data_ptr(), pd["z"].data_ptr(), pd["w"].data_ptr(), -1, *geo,
                    PP([d[k] for k in order])]
            name = "ccl_deposit_scalar"
        if use_lo:
            call(name + "_lo", *args, *ld, S())
        else:
            call(name, *args, S())
        errs.append(max(np.abs(to64(host(d[k])) - ref[k]).max() / np.abs(ref[k] - f0[k]).max()
                        for k in order))
    assert errs[0] < 2e-5 and errs[1] > 10 * errs[0], errs


@pytest.mark.parametrize("M", [0, 1])
def test_gather_push_cells_fp32_low_parts(cuda, port, M):
    """The tiled FP32 gather + push with compensated coordinates at x ~ -1e4:
    momentum increments within 5e-5 of the FP64 oracle's on the double
    coordinates, from hi alone at least 10x further off."""
    rng = np.random.default_rng(70 + M)
    g = geom(128, 32, Xmin=-10020.0, Xmax=-10000.0)
    q, lo, p = _split(particles(rng, 50000, g, boundaries=False))
    _, _, off, srt = oracle_sort(port, p, g)
    np_stay = int(off[-2])
    names = ["E" + c for c in "xyz"] + ["B" + c for c in "xyz"]
    f = {k: to64(to32(v)) for k, v in fields(rng, g["Nr"], g["Nx"], M, names).items()}
    order = [n + "_m" + str(m) for m in range(M + 1) for n in names]
    ref = {k: p[k].copy() for k in ("px", "py", "pz", "g_inv")}
    fp = 0.37
    geo = (g["Nx"], g["Xmin"], g["dx_inv"], g["Nr"], g["Rmin"], g["dr_inv"])
    port.gather_and_push(M, p["x"], p["y"], p["z"], ref["px"], ref["py"], ref["pz"], ref["g_inv"],
                         srt, fp, p["x"].size, np_stay, *geo, [f[k] for k in order])
    fd = [dev(to32(f[k])) for k in order]
    nst = torch.tensor([np_stay], dtype=torch.int32, device="cuda")
    ld = [dev(lo[k]).data_ptr() for k in ("x", "y", "z")]
    errs = []
    for use_lo in (True, False):
        pd = {k: dev(v) for k, v in q.items()}
        args = [CCL_F32, M, p["x"].size, pd["x"].data_ptr(), pd["y"].data_ptr(),
                pd["z"].data_ptr(), pd["px"].data_ptr(), pd["py"].data_ptr(), pd["pz"].data_ptr(),
                pd["g_inv"].data_ptr(), dev(srt).data_ptr(), dev(off).data_ptr(), nst.data_ptr(),
                fp, *geo, PP(fd)]
        if use_lo:
            call("ccl_gather_push_cells_lo", *args, *ld, S())
        else:
            call("ccl_gather_push_cells", *args, S())
        errs.append(max(np.abs(to64(host(pd[k])) - ref[k]).max() / np.abs(ref[k] - p[k]).max()
                        for k in ("px", "py", "pz")))
    assert errs[0] < 5e-5 and errs[1] > 10 * errs[0], errs


def test_low_parts_rejected_for_fp64(cuda):
    lib = _lib.load()
    t = torch.zeros(64, dtype=torch.float64, device="cuda")
    P = t.data_ptr()
    arr = (C.c_void_p * 1)(P)
    rc = lib.ccl_deposit_scalar_lo(CCL_F64, 0, P, P, P, P, P, P, -1, 16, 0.0, 1.0, 8, 0.0, 1.0,
                                   arr, P, P, P, S())
    assert rc != 0 and b"FP32" in lib.ccl_last_error()


# ------------------------------------------------------------------- spectral
def cplx(rng, *shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def test_psatd_bit_exact(cuda, port):
    rng = np.random.default_rng(40)
    n = 63 * 512
    f = [cplx(rng, n) for _ in range(15)]
    c1, c2, c3 = rng.uniform(-1, 1, n), rng.uniform(-3, 3, n), rng.uniform(0.01, 2, n)
    d = [dev(a) for a in f]
    ref = [a.copy() for a in f]
    port.advance_e_g_m(1 / 0.031, c1, c2, c3, ref)
    call("ccl_psatd_advance", CCL_F64, n, 1 / 0.031, dev(c1).data_ptr(), dev(c2).data_ptr(),
         dev(c3).data_ptr(), PP(d), S())
    for i in range(6):
        np.testing.assert_array_equal(host(d[i]), ref[i])


@pytest.mark.parametrize("sources_only", [False, True])
def test_psatd_split_fp32(cuda, port, sources_only):
    """The FP32 form's update (cancellation-free coefficients) against the
    oracle's FP64 advance_e_g_m on the same FP32-representable inputs, over
    w dt from 1e-3 (long waves) to 3: within 1e-6 of each output's norm,
    also for the source response alone (E = G = 0), whose long-wave part
    the reference's grouping would keep to 1-2 digits in FP32."""
    from chimeracl_gb300.methods.solver_methods_cu import psatd_split_coefficients
    rng = np.random.default_rng(42)
    n, dt = 63 * 512, 0.039
    w = np.exp(rng.uniform(np.log(1e-3), np.log(3.0), n)) / dt
    f = [cplx(rng, n).astype(np.complex64).astype(np.complex128) for _ in range(15)]
    if sources_only:
        for k in range(6):
            f[k][:] = 0
    ref = [a.copy() for a in f]
    port.advance_e_g_m(1 / dt, np.cos(w * dt), np.sin(w * dt) * w, 1 / w ** 2, ref)
    coef = dev(psatd_split_coefficients(w, dt).astype(np.float32))
    d = [dev(a.astype(np.complex64)) for a in f]
    call("ccl_psatd_advance_split", CCL_F32, n, coef.data_ptr(), PP(d), S())
    for i in range(6):
        got = host(d[i]).astype(np.complex128)
        assert np.linalg.norm(got - ref[i]) <= 1e-6 * np.linalg.norm(ref[i]), i


def test_elementwise_bit_exact(cuda, port):
    rng = np.random.default_rng(41)
    nr, nx = 31, 200
    x, y, z = cplx(rng, nr, nx), cplx(rng, nr, nx), cplx(rng, nr, nx)
    b = rng.normal(size=nx)
    r = rng.normal(size=(nr, nx))
    a, bb = 0.3 - 1.7j, -2.1 + 0.4j
    n = nr * nx
    for op in ("append", "zpaxz", "axpbyz", "mult", "abdot", "cast", "phase", "m1", "edges"):
        zr = z.copy()
        zd = dev(z)
        if op == "append":
            port.append_c2c(zr, x)
            call("ccl_append_c2c", CCL_F64, n, zd.data_ptr(), dev(x).data_ptr(), S())
        elif op == "zpaxz":
            port.zpaxz(zr, a, x)
            call("ccl_zpaxz", CCL_F64, n, zd.data_ptr(), a.real, a.imag, dev(x).data_ptr(), S())
        elif op == "axpbyz":
            port.axpbyz(a, x, bb, y, zr)
            call("ccl_axpbyz", CCL_F64, n, a.real, a.imag, dev(x).data_ptr(), bb.real, bb.imag,
                 dev(y).data_ptr(), zd.data_ptr(), S())
        elif op == "mult":
            port.mult_elementwise(r, zr)
            call("ccl_mult_elementwise", CCL_F64, n, dev(r).data_ptr(), zd.data_ptr(), S())
        elif op == "abdot":
            port.ab_dot_x(a, b, x, zr)
            call("ccl_ab_dot_x", CCL_F64, nr, nx, a.real, a.imag, dev(b).data_ptr(),
                 dev(x).data_ptr(), zd.data_ptr(), S())
        elif op == "cast":
            out_r = np.empty((nr, nx))
            port.cast_c2d(x, out_r)
            od = torch.empty((nr, nx), dtype=torch.float64, device="cuda")
            call("ccl_cast_c2d", CCL_F64, n, dev(x).data_ptr(), od.data_ptr(), S())
            np.testing.assert_array_equal(host(od), out_r)
            continue
        elif op == "phase":
            phs = np.exp(1j * rng.uniform(0, 6, nx))
            port.multiply_by_phase(zr, phs)
            call("ccl_multiply_by_phase", CCL_F64, nr, nx, zd.data_ptr(), dev(phs).data_ptr(), S())
        elif op == "m1":
            port.get_m1(zr, x, nx)
            call("ccl_get_m1", CCL_F64, nr, nx, zd.data_ptr(), dev(x).data_ptr(), S())
        elif op == "edges":
            prof = rng.uniform(0, 1, 40)
            port.profile_edges(zr, prof, nx, 40)
            call("ccl_profile_edges", CCL_F64, 1, nr, nx, zd.data_ptr(), dev(prof).data_ptr(), 40,
                 S())
        np.testing.assert_array_equal(host(zd), zr, err_msg=op)


def test_phase_table(cuda, port):
    nx = 512
    kx = 2 * np.pi * np.fft.fftfreq(nx, 0.078)
    for sign in (1, -1):
        ref = np.empty(nx, np.complex128)
        port.get_phase(ref, kx, -37.25, sign)
        d = torch.empty(nx, dtype=torch.complex128, device="cuda")
        call("ccl_phase", CCL_F64, nx, d.data_ptr(), dev(kx).data_ptr(), -37.25, sign, S())
        np.testing.assert_allclose(host(d), ref, rtol=0, atol=4e-16)


@pytest.mark.parametrize("nx", [64, 384, 512, 768, 900, 1024, 2000, 2048, 4096])
def test_fft_rows(cuda, nx):
    rng = np.random.default_rng(nx)
    nr = 37
    x = cplx(rng, nr, nx)
    xr = rng.normal(size=(nr + 1, nx))
    phs = np.exp(1j * rng.uniform(0, 6, nx))
    filt = rng.uniform(0, 1, (nr, nx))
    out = torch.empty((nr, nx), dtype=torch.complex128, device="cuda")
    # complex forward with filter
    call("ccl_fft_forward_rows", CCL_F64, nr, nx, dev(x).data_ptr(), nx, 0, out.data_ptr(),
         dev(phs).data_ptr(), dev(filt).data_ptr(), S())
    ref = np.fft.fft(x, axis=1) * phs * filt
    assert np.abs(host(out) - ref).max() <= FFT_TOL * np.abs(ref).max()
    # real forward from rows 1.. of a (nr+1, nx) real field, no filter
    xd = dev(xr)
    call("ccl_fft_forward_rows", CCL_F64, nr, nx, xd.data_ptr() + 8 * nx, nx, 1, out.data_ptr(),
         dev(phs).data_ptr(), None, S())
    ref = np.fft.fft(xr[1:].astype(np.complex128), axis=1) * phs
    assert np.abs(host(out) - ref).max() <= FFT_TOL * np.abs(ref).max()
    # backward, complex out and real-part out into rows 1..
    call("ccl_fft_backward_rows", CCL_F64, nr, nx, dev(x).data_ptr(), out.data_ptr(), nx, 0,
         dev(phs).data_ptr(), S())
    ref = np.fft.ifft(x * phs, axis=1)
    assert np.abs(host(out) - ref).max() <= FFT_TOL * np.abs(ref).max()
    call("ccl_fft_backward_rows", CCL_F64, nr, nx, dev(x).data_ptr(), xd.data_ptr() + 8 * nx, nx,
         1, dev(phs).data_ptr(), S())
    got = host(xd)
    np.testing.assert_array_equal(got[0], xr[0])
    assert np.abs(got[1:] - ref.real).max() <= FFT_TOL * np.abs(ref).max()


@pytest.mark.parametrize("nx", [512, 768, 1024, 2048, 4096])
def test_fft_rows_fp32(cuda, nx):
    """FP32 transforms (register-resident kernels at 512..4096) against
    numpy's FFT of the same FP32 data; bar 2e-6 of the largest magnitude."""
    rng = np.random.default_rng(nx + 1)
    nr = 21
    x = cplx(rng, nr, nx).astype(np.complex64)
    phs = np.exp(1j * rng.uniform(0, 6, nx)).astype(np.complex64)
    filt = rng.uniform(0, 1, (nr, nx)).astype(np.float32)
    out = torch.empty((nr, nx), dtype=torch.complex64, device="cuda")
    call("ccl_fft_forward_rows", CCL_F32, nr, nx, dev(x).data_ptr(), nx, 0, out.data_ptr(),
         dev(phs).data_ptr(), dev(filt).data_ptr(), S())
    ref = np.fft.fft(x.astype(np.complex128), axis=1) * phs * filt
    assert np.abs(host(out) - ref).max() <= 2e-6 * np.abs(ref).max()
    call("ccl_fft_backward_rows", CCL_F32, nr, nx, dev(x).data_ptr(), out.data_ptr(), nx, 0,
         dev(phs).data_ptr(), S())
    ref = np.fft.ifft(x.astype(np.complex128) * phs, axis=1)
    assert np.abs(host(out) - ref).max() <= 2e-6 * np.abs(ref).max()


def test_fft_unsupported_length(cuda):
    lib = _lib.load()
    t = torch.zeros(2 * 17 * 4, dtype=torch.float64, device="cuda")
    rc = lib.ccl_fft_forward_rows(CCL_F64, 2, 17 * 17, t.data_ptr(), 17 * 17, 0, t.data_ptr(),
                                  t.data_ptr(), None, S())
    assert rc == 3


@pytest.mark.parametrize("nx", [512, 2048])
@pytest.mark.parametrize("real_mode", [True, False])
def test_damp_rows(cuda, port, real_mode, nx):
    rng = np.random.default_rng(50 + real_mode)
    nr, nf = 31, 100
    spec = cplx(rng, nr, nx)
    rs0 = rng.normal(size=(nr + 1, nx)) if real_mode else cplx(rng, nr + 1, nx)
    kx = 2 * np.pi * np.fft.fftfreq(nx, 0.05)
    pp, pm = np.exp(1j * kx * -3.3), np.exp(-1j * kx * -3.3)
    prof = rng.uniform(0, 1, nf)
    # reference sequence: half backward, profile_edges, half forward
    b = np.fft.ifft(spec * pp, axis=1)
    rs_ref = rs0.copy()
    rs_ref[1:] = b.real if real_mode else b
    port.profile_edges(rs_ref, prof, nx, nf)
    spec_ref = np.fft.fft(rs_ref[1:].astype(np.complex128), axis=1) * pm
    sd, rd = dev(spec), dev(rs0)
    call("ccl_damp_rows", CCL_F64, nr, nx, sd.data_ptr(), rd.data_ptr(), int(real_mode),
         dev(pp).data_ptr(), dev(pm).data_ptr(), dev(prof).data_ptr(), nf, S())
    assert np.abs(host(rd) - rs_ref).max() <= FFT_TOL * np.abs(rs_ref).max()
    np.testing.assert_array_equal(host(rd)[0], rs_ref[0])
    assert np.abs(host(sd) - spec_ref).max() <= FFT_TOL * np.abs(spec_ref).max()


@pytest.mark.parametrize("m,k,ncols,cplx_,beta", [(63, 63, 1024, 1, 0.0), (255, 255, 4096, 1, 1.0),
                                                  (63, 63, 512, 0, 0.0), (100, 37, 130, 1, 1.0),
                                                  (511, 511, 256, 0, 1.0)])
def test_dht_gemm(cuda, m, k, ncols, cplx_, beta):
    rng = np.random.default_rng(m + k)
    A = rng.normal(size=(m, k))
    ldx = ncols + 6
    X = rng.normal(size=(k, ldx))
    Y0 = rng.normal(size=(m, ncols))
    al = (0.5 - 1.25j) if cplx_ else 0.75
    T = A @ X[:, :ncols]
    if cplx_:
        Tc = T[:, 0::2] + 1j * T[:, 1::2]
        Yc = Y0[:, 0::2] + 1j * Y0[:, 1::2]
        Rc = beta * Yc + al * Tc
        ref = np.empty_like(Y0)
        ref[:, 0::2], ref[:, 1::2] = Rc.real, Rc.imag
    else:
        ref = beta * Y0 + al * T
    Yd = dev(Y0)
    a = complex(al)
    call("ccl_dht_gemm", CCL_F64, 1, m, k, ncols, cplx_, PP([dev(A)]), PP([dev(X)]), ldx, PP([Yd]),
         ncols, a.real, a.imag, beta, S())
    assert np.abs(host(Yd) - ref).max() <= FFT_TOL * np.abs(ref).max()


def test_batched_transforms_match_single_calls(cuda):
    """One launch over several (field, mode) entries gives exactly what the
    per-entry launches give."""
    from chimeracl_gb300._lib import ints, longs
    rng = np.random.default_rng(60)
    nr, nx = 33, 256
    phs = dev(np.exp(1j * rng.uniform(0, 6, nx)))
    ins = [dev(cplx(rng, nr, nx)), dev(rng.normal(size=(nr, nx))), dev(cplx(rng, nr, nx))]
    real = [0, 1, 0]
    filt = [dev(rng.uniform(size=(nr, nx))), None, dev(rng.uniform(size=(nr, nx)))]
    outs_b = [torch.empty((nr, nx), dtype=torch.complex128, device="cuda") for _ in ins]
    call("ccl_fft_forward_batch", CCL_F64, 3, nr, nx, PP(ins), longs([nx] * 3), ints(real),
         PP(outs_b), phs.data_ptr(), PP(filt), S())
    for i in range(3):
        o = torch.empty_like(outs_b[i])
        call("ccl_fft_forward_rows", CCL_F64, nr, nx, ins[i].data_ptr(), nx, real[i],
             o.data_ptr(), phs.data_ptr(), None if filt[i] is None else filt[i].data_ptr(), S())
        torch.cuda.synchronize()
        assert torch.equal(o, outs_b[i])
    # backward: complex and real-part outputs
    bo = [torch.empty((nr, nx), dtype=torch.complex128, device="cuda"),
          torch.empty((nr, nx), dtype=torch.float64, device="cuda")]
    call("ccl_fft_backward_batch", CCL_F64, 2, nr, nx, PP([outs_b[0], outs_b[1]]), PP(bo),
         longs([nx, nx]), ints([0, 1]), phs.data_ptr(), S())
    for i, r in enumerate((0, 1)):
        o = torch.empty_like(bo[i])
        call("ccl_fft_backward_rows", CCL_F64, nr, nx, outs_b[i].data_ptr(), o.data_ptr(), nx, r,
             phs.data_ptr(), S())
        torch.cuda.synchronize()
        assert torch.equal(o, bo[i])
    # damping round trip on a real and a complex mode
    prof = dev(rng.uniform(size=40))
    specs = [dev(cplx(rng, nr, nx)), dev(cplx(rng, nr, nx))]
    rss = [dev(rng.normal(size=(nr + 1, nx))), dev(cplx(rng, nr + 1, nx))]
    s1 = [t.clone() for t in specs]
    r1 = [t.clone() for t in rss]
    call("ccl_damp_batch", CCL_F64, 2, nr, nx, PP(specs), PP(rss), ints([1, 0]), phs.data_ptr(),
         phs.data_ptr(), prof.data_ptr(), 40, S())
    for i, r in enumerate((1, 0)):
        call("ccl_damp_rows", CCL_F64, nr, nx, s1[i].data_ptr(), r1[i].data_ptr(), r,
             phs.data_ptr(), phs.data_ptr(), prof.data_ptr(), 40, S())
    torch.cuda.synchronize()
    for a, b in zip(specs + rss, s1 + r1):
        assert torch.equal(a, b)


def test_gemm_batch_per_entry_columns(cuda):
    from chimeracl_gb300._lib import ints, longs
    rng = np.random.default_rng(61)
    m = k = 63
    A = [dev(rng.normal(size=(m, k))), dev(rng.normal(size=(m, k)))]
    ncols = [200, 512]
    X = [dev(rng.normal(size=(k, n))) for n in ncols]
    Y = [torch.empty((m, n), dtype=torch.float64, device="cuda") for n in ncols]
    call("ccl_dht_gemm_batch", CCL_F64, 2, m, k, ints(ncols), 0, PP(A), PP(X), longs(ncols),
         PP(Y), longs(ncols), 1.0, 0.0, 0.0, S())
    for i in range(2):
        ref = host(A[i]) @ host(X[i])
        assert np.abs(host(Y[i]) - ref).max() <= FFT_TOL * np.abs(ref).max()


def test_copy_batch_aligned_misaligned_and_ragged(cuda):
    """ccl_copy_batch: 16-byte vector path where both arrays are 16-byte
    aligned, word by word otherwise; sizes with a ragged tail, empty arrays,
    and arrays of very different lengths in one launch."""
    from chimeracl_gb300._lib import longs
    rng = np.random.default_rng(71)
    words = [0, 1, 3, 4, 5, 1023, 4096 * 257 + 3, 17]
    offs = [0, 0, 1, 0, 2, 1, 0, 3]  # word offsets into the buffers (1..3: misaligned)
    srcs = [torch.from_numpy(rng.integers(0, 2**31, n + 8, dtype=np.int64).astype(np.int32)).cuda()
            for n in words]
    dsts = [torch.full((n + 8,), -7, dtype=torch.int32, device="cuda") for n in words]
    ptr = lambda t, o: t.data_ptr() + 4 * o  # noqa: E731
    call("ccl_copy_batch", len(words), longs([4 * n for n in words]),
         (C.c_void_p * len(words))(*[ptr(d, o) for d, o in zip(dsts, offs)]),
         (C.c_void_p * len(words))(*[ptr(s, o) for s, o in zip(srcs, offs)]), S())
    torch.cuda.synchronize()
    for n, o, s, d in zip(words, offs, srcs, dsts):
        hs, hd = host(s), host(d)
        np.testing.assert_array_equal(hd[o:o + n], hs[o:o + n])
        assert (hd[:o] == -7).all() and (hd[o + n:] == -7).all()  # nothing outside
