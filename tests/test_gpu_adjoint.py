"""The adjoint of the step (chimeracl_gb300/adjoint.py), through the C ABI.

Per operation, in FP64 on a small LPA run: each transpose against its
forward operation -- <lambda, A x> = <A^T lambda, x> for the linear ones
(PSATD update, spectral gradient and curl with their radial GEMMs, backward
and forward Fourier-Bessel transforms with the smoothing filter, edge
damping, deposit post-processing, ghost rows, align), and against a central
difference of the forward kernel along a random direction for the particle
ones (charge and current deposits, gather + Boris push, coordinate push).

Whole runs: the gradient of the wake loss with respect to the laser's a0,
waist R and focus x_foc and to density-profile knot values, against central
finite differences of the FP64 forward -- the FP64 adjoint on a 256 x 32
run of 20 steps (three window shifts with injection, four checkpoint
segments) within 1e-5 of the largest gradient, and the FP32 adjoint of the
mixed form (the differentiable run: 1024 x 128, 100 steps, checkpoint every
10) within 1e-3 (the bar the mixed form is held to; measured 6e-4, the FP32
trajectory's own difference from FP64)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

F64 = 0


def dot(a, b):
    """Real inner product of two lists of tensors (complex: Re conj(a) b)."""
    s = 0.0
    for x, y in zip(a, b):
        x = x.to(torch.complex128) if x.is_complex() else x.to(torch.float64)
        y = y.to(torch.complex128) if y.is_complex() else y.to(torch.float64)
        s += float((torch.conj(x) * y).real.sum()) if x.is_complex() else float((x * y).sum())
    return s


def rnd(t, g):
    if t.is_complex():
        return torch.complex(torch.randn(t.shape, generator=g, dtype=torch.float64),
                             torch.randn(t.shape, generator=g, dtype=torch.float64)).to(t)
    return torch.randn(t.shape, generator=g, dtype=torch.float64).to(t)


@pytest.fixture(scope="module")
def small_run(cuda):
    """An FP64 LPA run (64 x 16, M = 1) stepped 6 times (a window shift with
    injection at the first), with its adjoint helper prepared."""
    from chimeracl_gb300.adjoint import PICAdjoint
    from tests.lpa_setup import build_product, small_lpa
    cfg = small_lpa(Nx=64, Nr=16, M=1, a0=3.0, seed=11, steps=4)
    sol, eons, ions, loop = build_product(cfg, precision="fp64")
    for _ in range(6):
        loop.step()
    torch.cuda.synchronize()
    adj = PICAdjoint(loop, cfg["laser_in"])
    adj._prepare()
    return dict(sol=sol, eons=eons, ions=ions, loop=loop, adj=adj, cfg=cfg)


def _check(lhs, rhs, tol=1e-11):
    assert abs(lhs - rhs) <= tol * max(abs(lhs), abs(rhs), 1e-300), (lhs, rhs)


def test_psatd_adjoint(small_run):
    from chimeracl_gb300._lib import PP, call, stream
    from chimeracl_gb300.methods.solver_methods_cu import psatd_split_coefficients
    S, adj = small_run["sol"], small_run["adj"]
    g = torch.Generator().manual_seed(1)
    A = S.Args
    n = (A["Nr"] - 1) * A["Nx"]
    coef = torch.as_tensor(psatd_split_coefficients(A["w_m1"], A["dt"]), device="cuda")
    x = [rnd(adj._spec(), g) for _ in range(15)]
    y = [t.clone() for t in x]
    call("ccl_psatd_advance_split", F64, n, coef.data_ptr(), PP(y), stream())
    lam = [rnd(adj._spec(), g) for _ in range(6)]
    la = [t.clone() for t in lam] + [adj._spec() for _ in range(9)]
    call("ccl_psatd_adjoint", F64, n, coef.data_ptr(), None, PP(la), stream())
    _check(dot(lam, y[:6]), dot(la, x))


def test_grad_and_curl_adjoints(small_run):
    S, adj = small_run["sol"], small_run["adj"]
    D, M = S.DataDev, S.Args["M"]
    g = torch.Generator().manual_seed(2)
    # gradient: rho_fb -> dN1
    rho = [rnd(D["rho_fb_m%d" % m], g) for m in range(M + 1)]
    for m in range(M + 1):
        D["rho_fb_m%d" % m].copy_(rho[m])
    S.field_grad("rho", "dN1")
    out = [D["dN1" + c + "_fb_m%d" % m].clone() for m in range(M + 1) for c in "xyz"]
    lam = [rnd(t, g) for t in out]
    lrho = [adj._spec() for _ in range(M + 1)]
    adj._grad_adj([t.clone() for t in lam], lrho)
    _check(dot(lam, out), dot(lrho, rho))
    # curl with the Poisson factor: G_fb -> B_fb
    G = [rnd(D["G" + c + "_fb_m%d" % m], g) for m in range(M + 1) for c in "xyz"]
    for m in range(M + 1):
        for i, c in enumerate("xyz"):
            D["G" + c + "_fb_m%d" % m].copy_(G[3 * m + i])
    S.restore_B_fb()
    B = [D["B" + c + "_fb_m%d" % m].clone() for m in range(M + 1) for c in "xyz"]
    lB = [rnd(t, g) for t in B]
    adj.lG = [adj._spec() for _ in range(3 * (M + 1))]
    adj._rot_adj([t.clone() for t in lB])
    _check(dot(lB, B), dot(adj.lG, G))


def test_transform_adjoints(small_run):
    S, adj = small_run["sol"], small_run["adj"]
    D, A, M = S.DataDev, S.Args, S.Args["M"]
    g = torch.Generator().manual_seed(3)
    xmin = float(A["Xmin"])
    ppos, pneg = adj._phase(xmin, 1), adj._phase(xmin, -1)
    # backward: E_fb, B_fb -> E, B real rows 1..
    names = [f + c for m in range(M + 1) for f in "EB" for c in "xyz"]
    modes = [m for m in range(M + 1) for _ in range(6)]
    X = [rnd(D[n + "_fb_m%d" % m], g) for n, m in zip(names, modes)]
    for n, m, t in zip(names, modes, X):
        D[n + "_fb_m%d" % m].copy_(t)
    S.fb_transform(vects=["E", "B"], dir=1)
    rs = [D[n + "_m%d" % m][1:].clone() for n, m in zip(names, modes)]
    lEB = []
    for m in modes:
        t = adj._realsp(m)
        t[1:] = rnd(t[1:], g)
        lEB.append(t)
    adj.lE = [adj._spec() for _ in range(3 * (M + 1))]
    adj._backward_transform_adj([t.clone() for t in lEB], pneg)
    lB = adj.ws["lB"]
    spec_adj = [(adj.lE if n[0] == "E" else lB)[3 * m + "xyz".index(n[1])]
                for n, m in zip(names, modes)]
    _check(dot([t[1:] for t in lEB], rs), dot(spec_adj, X))
    # forward with the smoothing filter: rho real rows 1.. -> rho_fb (the
    # filter's transpose is the psatd / gradient transposes' job)
    rho = [rnd(D["rho_m%d" % m][1:], g) for m in range(M + 1)]
    for m in range(M + 1):
        D["rho_m%d" % m][1:] = rho[m]
    filt = [S._real_dev("SmoothingFilter_m%d" % m) for m in range(M + 1)]
    S.fb_transform(scals=["rho"], dir=0, filt=filt)
    sp = [D["rho_fb_m%d" % m].clone() for m in range(M + 1)]
    lsp = [rnd(t, g) for t in sp]
    lrs = [adj._realsp(m) for m in range(M + 1)]
    adj._forward_transform_adj([(m, lsp[m] * filt[m], lrs[m]) for m in range(M + 1)], ppos)
    _check(dot(lsp, sp), dot([t[1:] for t in lrs], rho))
    assert float(lrs[0][0].abs().max()) == 0.0


def test_damp_adjoint(small_run):
    S, adj = small_run["sol"], small_run["adj"]
    D, A, M = S.DataDev, S.Args, S.Args["M"]
    g = torch.Generator().manual_seed(4)
    xmin = float(A["Xmin"])
    names = [f + c + "_fb_m%d" % m for f in "EG" for m in range(M + 1) for c in "xyz"]
    x = [rnd(D[n], g) for n in names]
    for n, t in zip(names, x):
        D[n].copy_(t)
    S.damp_fields()
    y = [D[n].clone() for n in names]
    lam = [rnd(t, g) for t in y]
    k = 3 * (M + 1)
    adj.lE, adj.lG = [t.clone() for t in lam[:k]], [t.clone() for t in lam[k:]]
    adj._damp_adj(adj._phase(xmin, 1), adj._phase(xmin, -1))
    _check(dot(lam, y), dot(adj.lE + adj.lG, x))


def test_postproc_and_ghost_row_adjoints(small_run):
    from chimeracl_gb300._lib import PP, call, stream
    S, adj = small_run["sol"], small_run["adj"]
    D, A, M = S.DataDev, S.Args, S.Args["M"]
    g = torch.Generator().manual_seed(5)
    x = [rnd(D["rho_m%d" % m], g) for m in range(M + 1)]
    for m in range(M + 1):
        D["rho_m%d" % m].copy_(x[m])
    S.postproc_depose_scalar("rho")
    y = [D["rho_m%d" % m].clone() for m in range(M + 1)]
    lam = [rnd(t, g) for t in y]
    la = [t.clone() for t in lam]
    call("ccl_deposit_postproc_adjoint", F64, M, 1, PP(la), A["Nx"], A["Nr"],
         S._real_dev("dV_inv").data_ptr(), stream())
    _check(dot(lam, y), dot(la, x))
    # ghost rows of E (3 components over the modes)
    x = [rnd(D["E" + c + "_m%d" % m], g) for c in "xyz" for m in range(M + 1)]
    for i, (c, m) in enumerate((c, m) for c in "xyz" for m in range(M + 1)):
        D["E" + c + "_m%d" % m].copy_(x[i])
    S.preproc_project_vec("E")
    y = [D["E" + c + "_m%d" % m].clone() for c in "xyz" for m in range(M + 1)]
    lam = [rnd(t, g) for t in y]
    la = [t.clone() for t in lam]
    call("ccl_warp_axis_adjoint", F64, M, 3, PP(la), A["Nx"], stream())
    _check(dot(lam, y), dot(la, x))


def test_align_adjoint(small_run):
    from chimeracl_gb300._lib import PP, call, stream
    g = torch.Generator().manual_seed(6)
    n_pre, n = 1000, 700
    idx = torch.randperm(n_pre, generator=g)[:n].to(torch.int32).cuda()
    x = torch.randn(n_pre, generator=g, dtype=torch.float64).cuda()
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    call("ccl_align", F64, n, 1, PP([x]), PP([y]), idx.data_ptr(), stream())
    lam = torch.randn(n, generator=g, dtype=torch.float64).cuda()
    la = torch.zeros(n_pre, dtype=torch.float64, device="cuda")
    call("ccl_align_adjoint", F64, n, 1, PP([lam]), PP([la]), idx.data_ptr(), stream())
    _check(dot([lam], [y]), dot([la], [x]))


def _fd_dir(f, state, direc, eps):
    """Central difference of f (a list of tensors) along `direc`."""
    plus = f({k: v + eps * direc.get(k, 0) for k, v in state.items()})
    minus = f({k: v - eps * direc.get(k, 0) for k, v in state.items()})
    return [(a - b) / (2 * eps) for a, b in zip(plus, minus)]


def _particles(run):
    e = run["eons"]
    D = e.DataDev
    return {k: D[k].clone() for k in ("x", "y", "z", "px", "py", "pz", "g_inv", "w")}, e


def test_deposit_adjoints(small_run):
    """Charge and current deposits: the transpose against a central
    difference along a random direction of positions, momenta, g_inv and
    weights (the cell sort redone for every evaluation)."""
    from chimeracl_gb300._lib import PP, call, sort_workspace_bytes, stream
    S, adj = small_run["sol"], small_run["adj"]
    A, M = S.Args, S.Args["M"]
    st, e = _particles(small_run)
    n = int(e.Args["Np"])
    C = (A["Nx"] - 1) * (A["Nr"] - 1)
    gp = adj._gp(A["Xmin"])
    ws_b = sort_workspace_bytes(n, C)
    ws = torch.empty(ws_b, dtype=torch.uint8, device="cuda")

    def sort(p):
        i32 = lambda k: torch.empty(k, dtype=torch.int32, device="cuda")
        keys, cnt, off, si, ns = i32(n), i32(C + 1), i32(C + 2), i32(n), i32(1)
        call("ccl_index_sort", F64, n, p["x"].data_ptr(), p["y"].data_ptr(), p["z"].data_ptr(),
             gp[0], gp[1], gp[2], gp[3], gp[4], gp[5], keys.data_ptr(), cnt.data_ptr(),
             off.data_ptr(), si.data_ptr(), ns.data_ptr(), ws.data_ptr(), ws_b, stream())
        return si, off

    def deposit(vec):
        def f(p):
            si, off = sort(p)
            out = [adj._realsp(m) for m in range(M + 1) for _ in range(3 if vec else 1)]
            if vec:
                call("ccl_deposit_vector", F64, M, si.data_ptr(), off.data_ptr(),
                     *[p[k].data_ptr() for k in ("x", "y", "z", "px", "py", "pz", "g_inv", "w")],
                     -1, *gp, PP(out), stream())
            else:
                call("ccl_deposit_scalar", F64, M, si.data_ptr(), off.data_ptr(),
                     *[p[k].data_ptr() for k in ("x", "y", "z", "w")], -1, *gp, PP(out),
                     stream())
            return out
        return f

    g = torch.Generator().manual_seed(7)
    for vec in (False, True):
        direc = {k: torch.randn(n, generator=g, dtype=torch.float64).cuda() for k in st}
        direc["x"] *= A["dx"]
        direc["y"] *= A["dr"]
        direc["z"] *= A["dr"]
        fd = _fd_dir(deposit(vec), st, direc, 1e-7)
        lam = [rnd(t, g) for t in fd]
        L = adj._particle_adj(n, True)
        si, off = sort(st)
        u = [st[k].data_ptr() for k in ("px", "py", "pz", "g_inv")]
        call("ccl_deposit_adjoint", F64, int(vec), M, si.data_ptr(), off.data_ptr(),
             st["x"].data_ptr(), st["y"].data_ptr(), st["z"].data_ptr(), *u, st["w"].data_ptr(),
             -1, *gp, PP(lam), L["x"].data_ptr(), L["y"].data_ptr(), L["z"].data_ptr(),
             L["w"].data_ptr(), L["px"].data_ptr(), L["py"].data_ptr(), L["pz"].data_ptr(),
             L["g_inv"].data_ptr(), stream())
        keys = list(st) if vec else ["x", "y", "z", "w"]
        _check(dot(lam, fd), dot([L[k] for k in keys], [direc[k] for k in keys]), tol=1e-6)


def test_gather_push_adjoint(small_run):
    """Gather + Boris push: the transpose (particle and field adjoints)
    against a central difference of the forward along a random direction
    of positions, momenta and the gathered E, B."""
    from chimeracl_gb300._lib import PP, call, stream
    S, adj, e = small_run["sol"], small_run["adj"], small_run["eons"]
    A, D, M = S.Args, S.DataDev, S.Args["M"]
    for fld in ("E", "B"):
        S.preproc_project_vec(fld)
    F = [D[f + c + "_m%d" % m].clone() for m in range(M + 1) for f in "EB" for c in "xyz"]
    st, _ = _particles(small_run)
    n = int(e.Args["Np"])
    Dp = e.DataDev
    si, co, ns = Dp["sort_indx"], Dp["cell_offset"], Dp["Np_stay_dev"]
    gp = adj._gp(A["Xmin"])
    fp = float(e.Args["FactorPush"])
    g = torch.Generator().manual_seed(8)

    def push(p):
        u = {k: p[k].clone() for k in ("px", "py", "pz", "g_inv")}
        fl = [p["F%d" % i] for i in range(len(F))]
        call("ccl_gather_push", F64, M, n, p["x"].data_ptr(), p["y"].data_ptr(),
             p["z"].data_ptr(), u["px"].data_ptr(), u["py"].data_ptr(), u["pz"].data_ptr(),
             u["g_inv"].data_ptr(), si.data_ptr(), ns.data_ptr(), fp, *gp, PP(fl), stream())
        return [u["px"], u["py"], u["pz"], u["g_inv"]]

    state = {k: st[k] for k in ("x", "y", "z", "px", "py", "pz", "g_inv")}
    state.update({"F%d" % i: t for i, t in enumerate(F)})
    direc = {k: torch.randn(v.shape, generator=g, dtype=torch.float64).cuda().to(v.dtype)
             for k, v in state.items() if k != "g_inv"}
    direc["x"] *= A["dx"]
    direc["y"] *= A["dr"]
    direc["z"] *= A["dr"]
    fd = _fd_dir(push, state, direc, 1e-7)
    lam = [torch.randn(n, generator=g, dtype=torch.float64).cuda() for _ in range(4)]
    L = adj._particle_adj(n, True)
    for k, t in zip(("px", "py", "pz", "g_inv"), lam):
        L[k].copy_(t)
    lF = [torch.zeros_like(t) for t in F]
    call("ccl_gather_push_adjoint", F64, M, st["x"].data_ptr(), st["y"].data_ptr(),
         st["z"].data_ptr(), st["px"].data_ptr(), st["py"].data_ptr(), st["pz"].data_ptr(),
         si.data_ptr(), co.data_ptr(), ns.data_ptr(), fp, *gp, PP(F), PP(lF),
         L["x"].data_ptr(), L["y"].data_ptr(), L["z"].data_ptr(), L["px"].data_ptr(),
         L["py"].data_ptr(), L["pz"].data_ptr(), L["g_inv"].data_ptr(), stream())
    rhs = dot([L[k] for k in ("x", "y", "z", "px", "py", "pz")],
              [direc[k] for k in ("x", "y", "z", "px", "py", "pz")])
    rhs += dot(lF, [direc["F%d" % i] for i in range(len(F))])
    # the forward keeps g_inv of particles it does not push: their g_inv
    # adjoint passes through (the direction has no g_inv part)
    _check(dot(lam, fd), rhs, tol=1e-6)


def test_push_x_adjoint(small_run):
    from chimeracl_gb300._lib import call, stream
    st, e = _particles(small_run)
    n = int(e.Args["Np"])
    adj = small_run["adj"]
    g = torch.Generator().manual_seed(9)
    dt = float(e.Args["dt_2"])

    def push(p):
        x = {k: p[k].clone() for k in ("x", "y", "z")}
        call("ccl_push_x", F64, n, x["x"].data_ptr(), x["y"].data_ptr(), x["z"].data_ptr(),
             p["px"].data_ptr(), p["py"].data_ptr(), p["pz"].data_ptr(), p["g_inv"].data_ptr(),
             dt, stream())
        return [x["x"], x["y"], x["z"]]

    direc = {k: torch.randn(n, generator=g, dtype=torch.float64).cuda() for k in st}
    fd = _fd_dir(push, st, direc, 1e-6)
    lam = [torch.randn(n, generator=g, dtype=torch.float64).cuda() for _ in range(3)]
    L = adj._particle_adj(n, True)
    for k, t in zip("xyz", lam):
        L[k].copy_(t)
    call("ccl_push_x_adjoint", F64, n, st["px"].data_ptr(), st["py"].data_ptr(),
         st["pz"].data_ptr(), st["g_inv"].data_ptr(), L["x"].data_ptr(), L["y"].data_ptr(),
         L["z"].data_ptr(), L["px"].data_ptr(), L["py"].data_ptr(), L["pz"].data_ptr(),
         L["g_inv"].data_ptr(), dt, stream())
    keys = ("x", "y", "z", "px", "py", "pz", "g_inv")
    _check(dot(lam, fd), dot([L[k] for k in keys], [direc[k] for k in keys]), tol=1e-8)


# ----------------------------------------------------------------------
def _loss(problem, params, knots):
    from chimeracl_gb300.adjoint import build_problem_run
    run = build_problem_run(problem, params, knots)
    run["loop"].graphs = True
    for _ in range(problem["nsteps"]):
        run["loop"].step()
    torch.cuda.synchronize()
    return float(run["adjoint"].wake_loss(problem["loss_width"]))


def _fd_gradients(problem, params, knots, which_knots, rel=1e-6):
    """Central differences of the FP64 forward's loss.  The step is small:
    the loss is piecewise smooth in the parameters (every particle that
    crosses a cell face in between adds a kink of the linear shape
    functions), and steps of 1e-4 already average over such kinks (4e-4 of
    the gradient on the 1024 x 128 run), while at 1e-6 the differences
    settle on the derivative (the FP64 adjoint agrees to 1e-6)."""
    p64 = dict(problem, precision="fp64")
    g = []
    for i in range(3):
        h = rel * max(abs(params[i]), 1.0)
        a, b = params.copy(), params.copy()
        a[i] += h
        b[i] -= h
        g.append((_loss(p64, a, knots) - _loss(p64, b, knots)) / (2 * h))
    gk = []
    for k in which_knots:
        h = rel * abs(knots[k])
        a, b = knots.copy(), knots.copy()
        a[k] += h
        b[k] -= h
        gk.append((_loss(p64, params, a) - _loss(p64, params, b)) / (2 * h))
    return np.array(g), np.array(gk)


def _adjoint_gradients(problem, params, knots):
    from chimeracl_gb300.adjoint import PICLoss
    p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    k = torch.tensor(knots, dtype=torch.float64, requires_grad=True)
    loss = PICLoss.apply(p, k, problem)
    loss.backward()
    return float(loss.detach()), p.grad.numpy(), k.grad.numpy()


def test_adjoint_fp64_small_run_matches_finite_differences(cuda):
    """256 x 32, 20 steps with a window shift and injection every 8 (steps
    0, 8, 16) and a checkpoint every 6 (four segments, the last partial)."""
    from chimeracl_gb300.adjoint import differentiable_problem
    problem, params, knots = differentiable_problem(seed=3, nsteps=20, precision="fp64",
                                                    Nx=256, Nr=32, nknots=8, every=6)
    problem["frame_in"]["Steps"] = 8
    problem["loss_width"] = 25.0
    loss, gp, gk = _adjoint_gradients(problem, params, knots)
    assert loss > 0
    which = list(np.argsort(-np.abs(gk))[:3])
    fp, fk = _fd_gradients(problem, params, knots, which)
    scale = max(np.abs(fp).max(), np.abs(fk).max())
    err = max(np.abs(gp - fp).max(), np.abs(gk[which] - fk).max()) / scale
    assert err < 1e-5, (gp, fp, gk[which], fk, err)


def test_adjoint_mixed_config_run_matches_fp64_finite_differences(cuda):
    """The differentiable run: 1024 x 128, 100 FP32 steps (mixed form) with a
    checkpoint every 10; gradients w.r.t. a0, w0, x_foc and the four knots
    of largest gradient against central differences of the FP64 forward."""
    from chimeracl_gb300.adjoint import differentiable_problem
    problem, params, knots = differentiable_problem(seed=0)
    loss, gp, gk = _adjoint_gradients(problem, params, knots)
    which = list(np.argsort(-np.abs(gk))[:4])
    fp, fk = _fd_gradients(problem, params, knots, which)
    scale = max(np.abs(fp).max(), np.abs(fk).max())
    err = max(np.abs(gp - fp).max(), np.abs(gk[which] - fk).max()) / scale
    assert err < 1e-3, (gp, fp, gk[which], fk, err)
