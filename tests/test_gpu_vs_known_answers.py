"""The reference's two known-answer scripts through the product's public API
on the GPU (the same procedures run on the oracle in tests/test_oracle.py):
examples/test_transformer.py -- a deposited beam's forward + backward
Fourier-Bessel transform returns the deposit (1e-10 in FP64; 1e-4 in the
mixed form, whose two BF16x3 transforms each keep ~16 bits: a numpy
emulation of the split products on this deposit gives 1.6e-5, modes 0 and
1 together, the Hankel matrices' condition numbers being 23 and 12) -- and
examples/test_laser_veloc.py -- the PSATD propagation of a focused pulse
gives the analytic group-velocity correction, with the oracle's pinned
deviations reproduced to 1e-3 relative in FP64."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# the oracle's deviations (tests/test_oracle.py::test_known_answer_laser_group_velocity)
ORACLE_VELOCITY_ERRORS = (1.0390489878432e-04, 1.0728571893408624e-02)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-4)])
def test_fourier_bessel_round_trip(cuda, precision, tol):
    from chimeracl_gb300 import Communicator
    from chimeracl_gb300.particles import Particles
    from chimeracl_gb300.solver import Solver
    gi = dict(Xmin=-1.0, Xmax=1.0, Nx=256, Rmin=0, Rmax=1.0, Nr=64, M=1)
    comm = Communicator(precision=precision, seed=0)
    grid = Solver(dict(gi), comm)
    p = Particles(dict(gi), comm, seed=0)
    p.make_new_beam(dict(Np=50000, FullCharge=1, x_c=0.0, Lx=0.3, y_c=0.2, Ly=0.3, z_c=0.2,
                         Lz=0.3))
    p.add_new_particles()
    p.sort_parts(grid)
    p.align_parts()
    grid.depose_charge([p])
    D = grid.DataDev
    t0, t1 = D["rho_m0"].clone(), D["rho_m1"].clone()
    grid.fb_transform(scals=["rho"], dir=0)
    D["rho_m0"].zero_()
    D["rho_m1"].zero_()
    grid.fb_transform(scals=["rho"], dir=1)
    torch.cuda.synchronize()
    r0, r1 = (D["rho_m0"][1:] - t0[1:]).abs().max(), (D["rho_m1"][1:] - t1[1:]).abs().max()
    s0, s1 = t0[1:].abs().max(), t1[1:].abs().max()
    assert float(s0) > 0 and float(s1) > 0
    err = float(r0 / s0) + float(r1 / s1)
    assert err < tol, err


def test_laser_group_velocity_fp64(cuda):
    from chimeracl_gb300 import Communicator
    from chimeracl_gb300.laser import add_gausian_pulse
    from chimeracl_gb300.solver import Solver
    g = {"Xmin": -50.0, "Xmax": 50.0, "Rmax": 50.0}
    dx, dr, g["dt"] = 0.05, 0.3, 0.05
    g["Nx"] = int((g["Xmax"] - g["Xmin"]) / dx) // 2 * 2
    g["Nr"] = int(g["Rmax"] / dr) // 2 * 2 + 1
    g["M"] = 0
    laser = dict(k0=1.0, a0=1.0, x0=0, Lx=12.0, R=12.0, x_foc=20.0)
    s = Solver(g, Communicator(precision="fp64"))
    add_gausian_pulse(s, laser)
    x1, x2 = [], []
    Xg, Rg = s.Args["Xgrid"], s.Args["Rgrid"]
    for _ in range(100):
        s.push_fields()
        s.fb_transform(scals=["Ez"], dir=1)
        v = s.DataDev["Ez_m0"].cpu().numpy()
        Px = (Rg[1:, None] * v[1:, :] ** 2).sum(0)
        x1.append((Xg[None, :] * Px).sum() / Px.sum())
        Px = v[1, :] ** 2
        x2.append((Xg[None, :] * Px).sum() / Px.sum())
    errs = []
    for xs, fac in ((x1, 1.0), (x2, 2.0)):
        xs = np.array(xs)
        vn = 1 - (xs[1:] - xs[:-1]) / s.Args["dt"]
        vt = fac * (2.0 * np.pi * laser["R"]) ** -2
        errs.append(np.abs(vn - vt).mean() / vt)
    assert errs[0] < 1e-3 and errs[1] < 2e-2, errs
    np.testing.assert_allclose(errs, ORACLE_VELOCITY_ERRORS, rtol=1e-3)
