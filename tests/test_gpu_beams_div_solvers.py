"""Three parts of the reference's API beyond the single-species loop, through
the public API in FP64 against the oracle:

* ``field_div`` (transformer_methods_cl.py:135-183): the spectral divergence
  of a random vector field, every mode, within 1e-12 of the oracle's
  (M = 0, 1, 2);
* beam injection and normal momenta (particles_methods_cl.py:114-177):
  ``make_new_beam`` and a thermal ``make_new_domain`` draw the same seeded
  normal streams as the oracle, value for value; a beam species injected
  into a plasma run then steps with it, fields within 1e-12;
* several solvers in one loop (pic_loop.py:31-37, 80-140): a second solver on
  the same grid deposits the same species and pushes them again with its own
  fields, as the reference's loop does; both solvers' fields and the
  particles after 10 steps with two window shifts match the oracle run the
  same way.
"""
import copy

import numpy as np
import pytest
import torch

from tests.lpa_setup import build_oracle, build_product, compare_fields, small_lpa, to_np

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M", [0, 1, 2])
def test_field_div_matches_oracle(cuda, M):
    cfg = small_lpa(Nx=64, Nr=16, M=M, seed=5)
    sol, _, _, _ = build_product(cfg, precision="fp64")
    osol, _, _, _ = build_oracle(cfg)
    rng = np.random.default_rng(7)
    shape = (cfg["grid_in"]["Nr"] - 1, cfg["grid_in"]["Nx"])
    for m in range(M + 1):
        for c in "xyz":
            v = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
            k = "E" + c + "_fb_m%d" % m
            sol.DataDev[k].copy_(torch.from_numpy(v))
            osol.D[k][:] = v
    sol.field_div("E", "rho")
    osol.field_div("E", "rho")
    torch.cuda.synchronize()
    for m in range(M + 1):
        got, ref = to_np(sol.DataDev["rho_fb_m%d" % m]), osol.D["rho_fb_m%d" % m]
        assert np.abs(ref).max() > 0
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), m


def _beam_in():
    return dict(Np=20000, FullCharge=0.05, x_c=-20.0, Lx=1.0, y_c=0.0, Ly=1.5, z_c=0.0, Lz=1.5,
                px_c=50.0, dpx=2.0, py_c=0.0, dpy=0.3, pz_c=0.0, dpz=0.3)


def test_beam_and_thermal_injection_draws_match_oracle(cuda):
    from chimeracl_gb300 import Communicator
    from chimeracl_gb300.particles import Particles
    from oracle.kernels import get_kernels
    from oracle.pic_oracle import OSpecies
    K = get_kernels("port")
    base = dict(dx=0.1, dr=0.2, dt=0.1, charge=-1)
    p = Particles(dict(base), Communicator(precision="fp64"), seed=31)
    o = OSpecies(dict(base), K, seed=31)
    p.make_new_beam(_beam_in())
    o.make_new_beam(_beam_in())
    torch.cuda.synchronize()
    for k in ("x", "y", "z", "px", "py", "pz", "w"):
        np.testing.assert_array_equal(to_np(p.DataDev[k + "_new"]), o.D[k + "_new"], err_msg=k)
    np.testing.assert_allclose(to_np(p.DataDev["g_inv_new"]), o.D["g_inv_new"], rtol=1e-15)
    # a thermal plasma: normal momenta around a drift
    th = dict(base, Nppc=(2, 2, 4), dens=1e-3)
    p = Particles(copy.deepcopy(th), Communicator(precision="fp64"), seed=32)
    o = OSpecies(copy.deepcopy(th), K, seed=32)
    dom = dict(Xmin=-4.0, Xmax=0.0, Rmin=0.0, Rmax=2.0, px_c=0.1, dpx=0.01, dpy=0.02, dpz=0.03)
    p.make_new_domain(dict(dom))
    o.make_new_domain(dict(dom))
    torch.cuda.synchronize()
    for k in ("x", "y", "z", "w", "px", "py", "pz"):
        got, ref = to_np(p.DataDev[k + "_new"]), o.D[k + "_new"]
        assert got.shape == ref.shape and np.abs(ref).max() > 0, k
        # x, w exact; y, z within the injector's sin/cos ulps (CUDA's vs the
        # C library's); momenta exact (host draws)
        tol = 0.0 if k in ("x", "w", "px", "py", "pz") else 1e-15
        assert np.abs(got - ref).max() <= tol * np.abs(ref).max(), k
    np.testing.assert_allclose(to_np(p.DataDev["g_inv_new"]), o.D["g_inv_new"], rtol=1e-15)


def test_beam_in_plasma_steps_match_oracle(cuda):
    from chimeracl_gb300.particles import Particles
    from chimeracl_gb300.pic_loop import PIC_loop
    from oracle.pic_oracle import OLoop, OSpecies
    cfg = small_lpa(Nx=64, Nr=16, M=1, seed=9, a0=1.0)
    cfg["frame_in"] = None
    sol, e, i, loop = build_product(cfg, precision="fp64")
    osol, oe, oi, oloop = build_oracle(cfg)
    b_in = dict(cfg["eons_in"], dx=sol.Args["dx"], dr=sol.Args["dr"], dt=sol.Args["dt"])
    b_in.pop("Nppc")
    beam = Particles(copy.deepcopy(b_in), sol.comm, seed=77)
    obeam = OSpecies(copy.deepcopy(b_in), oe.K, seed=77)
    pin = dict(_beam_in(), x_c=-25.0, Np=4000)
    beam.make_new_beam(dict(pin))
    beam.add_new_particles()
    obeam.make_new_beam(dict(pin))
    obeam.add_new_particles()
    loop = PIC_loop([sol], [e, i, beam], [])
    oloop = OLoop([osol], [oe, oi, obeam], [])
    for _ in range(5):
        loop.step()
        oloop.step()
    torch.cuda.synchronize()
    assert compare_fields(sol, osol, dens=cfg["eons_in"]["dens"]) < 1e-12
    for k in ("x", "px", "pz"):
        got, ref = to_np(beam.DataDev[k]), obeam.D[k]
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), k


def test_two_solvers_in_one_loop_match_oracle(cuda):
    from chimeracl_gb300.pic_loop import PIC_loop
    from chimeracl_gb300.solver import Solver
    from oracle.pic_oracle import OGrid, OLoop
    cfg = small_lpa(Nx=64, Nr=16, M=1, seed=13, steps=4)
    sol, e, i, loop = build_product(cfg, precision="fp64")
    osol, oe, oi, oloop = build_oracle(cfg)
    sol2 = Solver(copy.deepcopy(cfg["grid_in"]), sol.comm)
    osol2 = OGrid(copy.deepcopy(cfg["grid_in"]), oe.K)
    loop = PIC_loop([sol, sol2], [e, i], loop.frames)
    oloop = OLoop([osol, osol2], [oe, oi], oloop.frames)
    for _ in range(10):
        loop.step()
        oloop.step()
    torch.cuda.synchronize()
    dens = cfg["eons_in"]["dens"]
    assert compare_fields(sol, osol, dens=dens) < 1e-11
    assert compare_fields(sol2, osol2, dens=dens) < 1e-11
    assert e.Args["Np"] == oe.Args["Np"]
    for k in ("x", "y", "px", "pz"):
        got, ref = to_np(e.DataDev[k]), oe.D[k]
        assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max(), k
