"""Whole PIC steps through the public API (Solver / Particles / Frame /
PIC_loop on the CUDA library) against the oracle running the reference's
step on the same seeded inputs.

Bars (plain FP64 form): sort keys, counts and order identical; fields after
one step within 1e-12 of their physical scale (tests.lpa_setup.field_floor:
arrays that are rounding residue of a neutral plasma are measured against
the magnitude of the quantity, not against their own noise); after 25 steps
(one window shift + injection, then a second at step 20) within 1e-10."""
import numpy as np
import pytest
import torch

from tests.lpa_setup import build_oracle, build_product, compare_fields, rel_err, small_lpa, to_np

pytestmark = pytest.mark.gpu


def _particles_equal(p, op, tol=0.0):
    for k in op.D:
        if k.endswith("_new") or k in ("indx_in_cell", "sum_in_cell", "cell_offset", "sort_indx"):
            continue
        e = rel_err(to_np(p.DataDev[k]), op.D[k])
        assert e <= tol, (k, e)


def _sort_equal(p, op):
    for k in ("indx_in_cell", "sum_in_cell", "cell_offset", "sort_indx"):
        np.testing.assert_array_equal(to_np(p.DataDev[k]).view(np.uint32), op.D[k], err_msg=k)


@pytest.mark.parametrize("M", [0, 1, 2])
def test_one_step_fp64(cuda, M):
    cfg = small_lpa(Nx=128, Nr=32, M=M, seed=11 + M)
    sol, e, i, loop = build_product(cfg)
    osol, oe, oi, oloop = build_oracle(cfg)
    # identical starting state (the laser's spectral init runs through FFTs)
    dens = cfg["eons_in"]["dens"]
    assert compare_fields(sol, osol, dens=dens) < 1e-12
    # y, z of the injector come from CUDA's sin/cos vs the host libm: ulps
    _particles_equal(e, oe, tol=1e-15)
    loop.step()
    oloop.step()
    torch.cuda.synchronize()
    _sort_equal(e, oe)
    _sort_equal(i, oi)
    assert e.Args["Np"] == oe.Args["Np"] and e.Args["Np_stay"] == oe.Args["Np_stay"]
    worst = compare_fields(sol, osol, dens=dens)
    assert worst < 1e-12, worst
    _particles_equal(e, oe, tol=1e-12)


def test_25_steps_fp64_window(cuda):
    cfg = small_lpa(Nx=128, Nr=32, M=1, seed=5)
    sol, e, i, loop = build_product(cfg)
    osol, oe, oi, oloop = build_oracle(cfg)
    for _ in range(25):
        loop.step()
        oloop.step()
    torch.cuda.synchronize()
    assert e.Args["Np"] == oe.Args["Np"]
    _sort_equal(e, oe)
    worst = compare_fields(sol, osol, dens=cfg["eons_in"]["dens"])
    assert worst < 1e-10, worst
    _particles_equal(e, oe, tol=1e-10)
    assert sol.Args["Xmin"] == osol.Args["Xmin"]


def test_two_mobile_species_fp64(cuda):
    """Electrons and mobile ions (charge +1, mass 100, injected on the
    electrons) through 25 steps and two window shifts: both species' pushes
    (their own charge-to-mass factor), sorts, current and charge deposits and
    gathers against the oracle's loop over the same two species
    (pic_loop.py:73-142).  Bar 1e-8 of each array's magnitude: the
    injector's y, z differ from the oracle's by ulps (CUDA's sin/cos vs the
    host libm), and the a0 = 3 pulse grows that to ~1.4e-9 in the momenta
    over 25 steps; a wrong charge-to-mass factor or a species left out of a
    deposit or gather would differ at 1e-2 or more."""
    cfg = small_lpa(Nx=128, Nr=32, M=1, seed=31, a0=3.0)
    sol, e, i, loop = build_product(cfg, ion_mass=100.0)
    osol, oe, oi, oloop = build_oracle(cfg, ion_mass=100.0)
    for _ in range(25):
        loop.step()
        oloop.step()
    torch.cuda.synchronize()
    for p, op in ((e, oe), (i, oi)):
        assert p.Args["Np"] == op.Args["Np"]
        _sort_equal(p, op)
        _particles_equal(p, op, tol=1e-8)
    assert float(np.abs(to_np(i.DataDev["px"])).max()) > 1e-4  # the ions did move
    worst = compare_fields(sol, osol, dens=cfg["eons_in"]["dens"])
    assert worst < 1e-8, worst


def test_density_profile_injection(cuda):
    prof = [{"coord": "x", "points": [-1e4, -40.0, -25.0, 1e6], "values": [0.0, 0.0, 1.0, 1.0]}]
    cfg = small_lpa(Nx=96, Nr=24, M=1, seed=9, profiles=prof, steps=5)
    sol, e, i, loop = build_product(cfg)
    osol, oe, oi, oloop = build_oracle(cfg)
    for _ in range(7):
        loop.step()
        oloop.step()
    torch.cuda.synchronize()
    _sort_equal(e, oe)
    assert compare_fields(sol, osol, dens=cfg["eons_in"]["dens"]) < 1e-11
    _particles_equal(e, oe, tol=1e-11)


def test_graph_replay_matches_eager(cuda):
    """Steps between window shifts replayed as a CUDA graph give exactly the
    eager steps' result (same kernels, same inputs)."""
    cfg = small_lpa(Nx=128, Nr=32, M=1, seed=23, steps=10)
    runs = []
    for graphs in (False, True):
        sol, e, i, loop = build_product(cfg, precision="fp64")
        loop.graphs = graphs
        for _ in range(24):
            loop.step()
        torch.cuda.synchronize()
        runs.append((sol, e, loop))
    (s0, e0, l0), (s1, e1, l1) = runs
    assert l1.graph_replays >= 18 and l1.graph_captures >= 2
    for k, v in s0.DataDev.items():
        if isinstance(v, torch.Tensor) and not k.startswith(("_", "buff_fb", "phs", "fld_buff")):
            assert torch.equal(v, s1.DataDev[k]), k
    for k in ("x", "y", "z", "px", "py", "pz", "g_inv", "w"):
        assert torch.equal(e0.DataDev[k], e1.DataDev[k]), k


class _Host:
    """numpy view of a product object for the oracle's diagnostics()."""

    def __init__(self, obj):
        self.Args = obj.Args
        self.D = {k: to_np(v) for k, v in obj.DataDev.items() if isinstance(v, torch.Tensor)}


def test_full_run_diagnostics_fp64(cuda):
    """The 512 x 64, M = 1 configuration (about 0.5M electrons, a0 = 2 laser,
    moving window) for 200 steps -- ten window shifts with injection --
    through the public API, through the oracle and in the committed run of
    the reference's own kernels: field energy, on-axis Ez wake amplitude and
    electron kinetic energy within 1e-6 relative."""
    from oracle.pic_oracle import diagnostics
    cfg = small_lpa(Nx=512, Nr=64, M=1, seed=21)
    sol, e, i, loop = build_product(cfg)
    osol, oe, oi, oloop = build_oracle(cfg)
    for _ in range(200):
        loop.step()
        oloop.step()
    torch.cuda.synchronize()
    assert e.Args["Np"] == oe.Args["Np"]
    got = diagnostics(_Host(sol), [_Host(e)])
    ref = diagnostics(osol, [oe])
    for k in ref:
        err = abs(got[k] / ref[k] - 1.0)
        assert err < 1e-6, (k, got[k], ref[k], err)
    # the same run of the reference's own kernels (committed fixture)
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "lpa_m1_512x64_200steps.npz"))
    assert e.Args["Np"] == int(g["count:Np"])
    for k in ref:
        err = abs(got[k] / float(g["diag:" + k]) - 1.0)
        assert err < 1e-6, (k, got[k], float(g["diag:" + k]), err)

