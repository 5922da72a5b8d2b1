"""Host-side logic of the product (CPU only): grid geometry, spectral axes,
Hankel matrices, PSATD coefficients and damping profile are built exactly as
the oracle builds them; the lazy Args container; injector draws."""
import copy

import numpy as np
import pytest

from oracle import pic_oracle as po


class _Stub:
    pass


def product_setup(cfg):
    from chimeracl_gb300.grid import Grid
    from chimeracl_gb300.methods.solver_methods_cu import SolverMethodsCU
    from chimeracl_gb300.solver import Solver
    from chimeracl_gb300.transformer import Transformer
    s = _Stub()
    Grid._process_configs(s, copy.deepcopy(cfg))
    if "DampCells" in cfg:
        SolverMethodsCU._init_field_damping(s)
    Transformer._make_spectral_axes(s)
    Transformer._make_DHT(s)
    Solver._make_ms_coefficients(s)
    return s.Args


@pytest.mark.parametrize("M,Nx,Nr", [(0, 64, 17), (1, 128, 32), (2, 96, 24)])
def test_setup_matches_oracle(M, Nx, Nr):
    cfg = dict(Xmin=-30.0, Xmax=0.0, Nx=Nx, Rmin=0.0, Rmax=15.0, Nr=Nr, M=M, DampCells=8)
    A = product_setup(cfg)
    O = po.OGrid(copy.deepcopy(cfg), K=object()).Args
    for k, v in O.items():
        if isinstance(v, (np.ndarray, float, int)) and k in A:
            np.testing.assert_array_equal(np.asarray(A[k]), np.asarray(v), err_msg=k)


def test_dht_matrices_invert():
    A = product_setup(dict(Xmin=-1.0, Xmax=1.0, Nx=32, Rmin=0.0, Rmax=1.0, Nr=64, M=1))
    for m in (0, 1):
        I = A["DHT_m%d" % m] @ A["DHT_inv_m%d" % m]
        assert np.abs(I - np.eye(I.shape[0])).max() < 1e-12


@pytest.mark.parametrize("real", ["float64", "float32"])
def test_psatd_coefficients_per_precision(real):
    """FP64 fields keep the reference's three coefficient arrays alone; FP32
    fields also get the eight cancellation-free ones, in float32."""
    import torch

    from chimeracl_gb300.grid import Grid
    from chimeracl_gb300.methods.solver_methods_cu import psatd_split_coefficients
    from chimeracl_gb300.solver import Solver
    from chimeracl_gb300.transformer import Transformer
    s = _Stub()
    s.comm = _Stub()
    s.comm.real = getattr(torch, real)
    Grid._process_configs(s, dict(Xmin=-20.0, Xmax=0.0, Nx=64, Rmin=0.0, Rmax=10.0, Nr=17,
                                  M=1))
    Transformer._make_spectral_axes(s)
    Transformer._make_DHT(s)
    Solver._make_ms_coefficients(s)
    A = s.Args
    for m in (0, 1):
        w, dt = A["w_m%d" % m], A["dt"]
        np.testing.assert_array_equal(A["MxSlv_cos(wdt)_m%d" % m], np.cos(w * dt))
        key = "MxSlv_split_m%d" % m
        if real == "float64":
            assert key not in A
        else:
            assert A[key].dtype == np.float32 and A[key].shape == w.shape + (8,)
            np.testing.assert_array_equal(A[key], psatd_split_coefficients(w, dt).astype(np.float32))
            assert key in A["dont_keep"]


def test_lazy_args():
    from chimeracl_gb300.methods.generic_methods_cu import ArgsDict, LazyScalar

    class T:
        def item(self):
            return 41

    a = ArgsDict(Np=3)
    dict.__setitem__(a, "Np_stay", LazyScalar(T()))
    assert a["Np_stay"] == 41 and a.get("Np_stay") == 41 and a["Np"] == 3
    assert type(dict.__getitem__(a, "Np_stay")) is int
    # a float read back lazily (the injector's right limit)
    dict.__setitem__(a, "right_lim", LazyScalar(T(), cast=float))
    assert a["right_lim"] == 41.0 and type(dict.__getitem__(a, "right_lim")) is float


def test_injector_draws_match_oracle():
    """The product draws the theta jitter and momenta from the same seeded
    PCG64 stream, in the same order, as the oracle."""
    rng_p = np.random.Generator(np.random.PCG64(5))
    rng_o = po.make_rng(5)
    th_p = 0 + (2 * np.pi - 0) * rng_p.random(100)
    th_o = 0.0 + (2 * np.pi - 0.0) * rng_o.random(100)
    np.testing.assert_array_equal(th_p, th_o)


class _FrameSpecies:
    """Stub species for Frame.inject_plasma: records the injection domain."""

    def __init__(self, x, x_lo=None):
        import torch
        self.Args = {"Np": len(x), "Nppc": np.array([2, 1, 4]), "ddx": 0.25, "right_lim": 0.0}
        self.DataDev = {"x": torch.tensor(x, dtype=torch.float32)}
        if x_lo is not None:
            self.DataDev["x_lo"] = torch.tensor(x_lo, dtype=torch.float32)
        self.comm = None
        self.domains = []

    def make_new_domain(self, dom, density_profiles=None):
        self.domains.append(dict(dom))

    def add_new_particles(self, source=None):
        pass

    def free_added(self):
        pass

    def sort_parts(self, grid):
        pass

    def align_parts(self):
        pass


@pytest.mark.parametrize("compensated", [False, True])
def test_injector_right_limit(compensated):
    """right_lim = max x of the last Nppc+1 particles + ddx/2 (frame.py:58-64),
    read lazily at the next shift; with compensated coordinates from x + x_lo
    in double."""
    from chimeracl_gb300.frame import Frame
    from chimeracl_gb300.methods.generic_methods_cu import ArgsDict
    x = np.float32(np.linspace(-3.0, 7.3, 12))
    lo = np.float32(np.spacing(x) * 0.25)
    sp = _FrameSpecies(x, lo if compensated else None)
    sp.Args = ArgsDict(sp.Args)
    grid = _Stub()
    grid.Args = {"Xmax": 8.0, "Rmin": 0.0, "Rmax": 4.0}
    fr = Frame({"Steps": 2, "Velocity": 1.0, "dt": 0.5})
    fr.inject_plasma([sp], grid)
    want = float(x[-9:].astype(np.float64).max())
    if compensated:
        want = float((x[-9:].astype(np.float64) + lo[-9:].astype(np.float64)).max())
    assert sp.Args["right_lim"] == want + 0.125
    fr.inject_plasma([sp], grid)  # the next shift starts there
    assert sp.domains[-1]["Xmin"] == want + 0.125


def test_injector_right_limit_fp32_uses_the_lattice_value():
    """FP32 coordinates: where the maximum of the last particles is the FP32
    value of the slab's last column, right_lim is that column's double value
    + ddx/2; otherwise (a particle moved past it) the FP32 maximum's."""
    from chimeracl_gb300.frame import Frame
    from chimeracl_gb300.methods.generic_methods_cu import ArgsDict
    c = -0.1 + 7.0 / 3.0  # a lattice x that FP32 does not hold exactly
    assert float(np.float32(c)) != c
    cols = [c, c - 0.125, c - 0.25, c - 0.375]  # last column first
    grid = _Stub()
    grid.Args = {"Xmax": 8.0, "Rmin": 0.0, "Rmax": 4.0}
    for case in ("last", "dropped", "moved"):
        x = np.float32(np.linspace(-3.0, 1.0, 12))
        x[-1] = {"last": np.float32(c), "dropped": np.float32(cols[2]),
                 "moved": np.float32(c + 0.01)}[case]
        sp = _FrameSpecies(x)
        sp.Args = ArgsDict(sp.Args)
        sp.Args["_inj_last_x"] = cols
        fr = Frame({"Steps": 2, "Velocity": 1.0, "dt": 0.5})
        fr.inject_plasma([sp], grid)
        want = {"last": c, "dropped": cols[2], "moved": float(np.float32(c + 0.01))}[case]
        assert sp.Args["right_lim"] == want + 0.125, case


@pytest.mark.parametrize("nppc", [(2, 2, 4), (2, 1, 4)])
def test_fp64_right_limits_are_injector_columns(nppc):
    """The premise of the FP32 forms' right limit, on the oracle's FP64 runs
    (a0 = 3 laser, moving window, five shifts): after each injection, sort
    and align, the largest x among the last Nppc + 1 particles -- what
    right_lim is formed from -- is exactly one of the injector's
    last-column values as the product computes them."""
    from chimeracl_gb300.methods.particles_methods_cu import injector_last_columns
    from tests.lpa_setup import build_oracle, small_lpa
    cfg = small_lpa(Nx=128, Nr=16, M=1, nppc=nppc, a0=3.0, steps=10, seed=7)
    osol, oe, oi, oloop = build_oracle(cfg)
    seen = []
    cand = {}
    make, align = oe.make_new_domain, oe.align_parts

    def make_new_domain(pin, density_profiles=None):
        n = int(np.ceil((pin["Xmax"] - pin["Xmin"]) / oe.Args["dx"]) + 1)
        Xg = pin["Xmin"] + oe.Args["dx"] * np.arange(n)
        cand["x"] = injector_last_columns(Xg, int(oe.Args["Nppc"][0]))
        return make(pin, density_profiles=density_profiles)

    def align_parts():
        align()
        k = int(np.prod(oe.Args["Nppc"]) + 1)
        seen.append((float(oe.D["x"][-k:].max()), list(cand["x"])))

    oe.make_new_domain, oe.align_parts = make_new_domain, align_parts
    for _ in range(41):
        oloop.step()
    assert len(seen) == 5
    for x_max, xs in seen:
        assert x_max in xs, (x_max, xs)


class _TwoHalfSpecies(_FrameSpecies):
    """Stub species with the two-half align: logs the order of the calls."""

    def __init__(self, name, log, x):
        super().__init__(x)
        self.name, self.log = name, log

    def sort_parts(self, grid):
        self.log.append(("sort", self.name))

    def align_begin(self):
        self.log.append(("align_begin", self.name))

    def align_end(self):
        self.log.append(("align_end", self.name))

    def align_parts(self):
        raise AssertionError("the shift aligns in two halves when every species can")


def test_shift_queues_every_align_before_reading_any_count():
    """At a window shift every species is sorted and its align queued
    before the first in-window count is read (align_end)."""
    from chimeracl_gb300.frame import Frame
    from chimeracl_gb300.methods.generic_methods_cu import ArgsDict
    log = []
    sps = [_TwoHalfSpecies(n, log, np.float32(np.linspace(-3.0, 7.3, 12))) for n in "ei"]
    for sp in sps:
        sp.Args = ArgsDict(sp.Args)
    grid = _Stub()
    grid.Args = {"Xmax": 8.0, "Rmin": 0.0, "Rmax": 4.0}
    Frame({"Steps": 2, "Velocity": 1.0, "dt": 0.5}).inject_plasma(sps, grid)
    kinds = [k for k, _ in log]
    assert kinds == ["sort", "sort", "align_begin", "align_begin", "align_end", "align_end"]
    assert [n for k, n in log if k == "align_end"] == ["e", "i"]


def test_tail_limit_is_the_device_formula():
    """TailLimit (host double arithmetic on a copy of the tail) equals the
    torch formula it replaces: max of x (+ x_lo) in double over the last
    Nppc+1 particles, for FP32 the snap to a candidate column's double value
    when the FP32 maximum is that column's rounding, + ddx/2."""
    import torch
    from chimeracl_gb300.frame import TailLimit
    rng = np.random.default_rng(3)
    for trial in range(200):
        n = int(rng.integers(1, 30))
        nppc = int(rng.integers(1, 12))
        x = np.float32(rng.uniform(-5, 5, n))
        comp = trial % 3 == 1
        lo = np.float32(np.spacing(x) * rng.uniform(-0.5, 0.5, n)) if comp else None
        cand = None
        if trial % 3 == 2:
            cand = list(rng.uniform(-5, 5, 4))
            if trial % 2:  # make the tail's maximum one candidate's FP32 rounding
                x[-1] = np.float32(max(np.float64(x[-nppc:].max()) + 1.0, cand[1]))
                cand[1] = float(x[-1]) + 1e-9 * rng.uniform(-1, 1)
                x[-1] = np.float32(cand[1])
        half = 0.5 * float(rng.uniform(0.01, 0.5))
        xt, lt = torch.tensor(x), (torch.tensor(lo) if comp else None)
        got = TailLimit(xt, lt, nppc, half, cand).resolve()
        tail = xt[-nppc:].to(torch.float64)
        if comp:
            tail = tail + lt[-nppc:].to(torch.float64)
        want = tail.max()
        if cand is not None:
            c = torch.tensor(cand, dtype=torch.float64)
            same = xt[-nppc:].max() == c.to(torch.float32)
            first = torch.argmax(same.to(torch.int32))
            want = torch.where(same.any(), c[first], want)
        assert got == float(want + half), trial
