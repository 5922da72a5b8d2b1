"""The astigmatic laser term (m = 2; the 4096 x 512 run's 20% component) in
the oracle's laser set-up, on the CPU: with the focus at the pulse the
spectral round trip returns Ez_m2 = -(a2/2) (r/R)^2 x the mode-0 profile,
the mode-0 fields are those of the plain laser bit for bit, the synthesised
field is the first-order expansion of the two-waist Gaussian, and fewer
than three modes are refused."""
import copy

import numpy as np
import pytest

from oracle import pic_oracle as po
from oracle.kernels import PortKernels

GRID = dict(Xmin=-40.0, Xmax=0.0, Nx=128, Rmin=0.0, Rmax=20.0, Nr=32, M=2, DampCells=16)
LASER = dict(k0=1.0, a0=2.0, x0=-10.0, Lx=3.0, R=6.0, x_foc=-10.0)


@pytest.fixture(scope="module")
def K():
    return PortKernels()


def _pulse(K, grid, **extra):
    sol = po.OGrid(copy.deepcopy(grid), K)
    po.add_gausian_pulse(sol, dict(LASER, **extra))
    return sol


def test_astigmatic_term_profile(K):
    a2 = 0.2
    sol = _pulse(K, GRID, astig=a2)
    plain = _pulse(K, GRID)
    D, P = sol.D, plain.D
    for f in ("E", "B"):
        for c in "xyz":
            np.testing.assert_array_equal(D[f + c + "_m0"], P[f + c + "_m0"])
    assert not np.any(P["Ez_m2"]) and np.any(D["Ez_m2"])
    r = sol.Args["Rgrid"][1:, None]
    want = -0.5 * a2 * (r / LASER["R"]) ** 2 * D["Ez_m0"][1:]
    scale = np.abs(D["Ez_m0"]).max()
    assert np.abs(D["Ez_m2"][1:] - want).max() < 1e-10 * scale
    # F_0 + 2 Re(F_2 e^{-2 i phi}) against exp(-r^2 (1 + a2 cos 2 phi)/R^2),
    # the two-waist Gaussian, to first order in a2
    for phi in (0.0, np.pi / 4, np.pi / 2):
        syn = D["Ez_m0"][1:] + 2 * np.real(D["Ez_m2"][1:] * np.exp(-2j * phi))
        env = np.exp(-(r / LASER["R"]) ** 2 * a2 * np.cos(2 * phi))
        exact = D["Ez_m0"][1:] * env
        assert np.abs(syn - exact).max() < 0.5 * a2 ** 2 * scale


def test_astigmatic_term_focused_has_energy_of_its_mode(K):
    """Focused 10 lambda0 away: the m = 2 pulse keeps the energy its profile
    carries (the propagator is unitary on the spectral fields)."""
    sol = _pulse(K, GRID, astig=0.2)
    foc = _pulse(K, GRID, astig=0.2, x_foc=0.0)
    e = [float((np.abs(s.D["Ez_fb_m2"]) ** 2 + np.abs(s.D["Gz_fb_m2"]) ** 2
                / s.Args["w_m2"] ** 2).sum()) for s in (sol, foc)]
    assert abs(e[1] / e[0] - 1) < 1e-12


def test_astigmatic_term_needs_three_modes(K):
    with pytest.raises(ValueError):
        _pulse(K, dict(GRID, M=1), astig=0.2)
