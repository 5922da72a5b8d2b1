"""The laser form of the 4096 x 512, m = 0..2 run through the public API
against the oracle: the 20% m = 2 astigmatic term set up on both sides
(M = 2), then one step."""
import pytest
import torch

from tests.lpa_setup import build_oracle, build_product, compare_fields, small_lpa
from tests.test_gpu_step import _particles_equal, _sort_equal

pytestmark = pytest.mark.gpu


def test_one_step_fp64_astigmatic_laser(cuda):
    """The laser form of the 4096 x 512, m = 0..2 run: a 20% m = 2
    astigmatic term (M = 2) set up on both sides, then one step -- fields within 1e-12
    of their physical scale, sort arrays identical, particles within 1e-12."""
    cfg = small_lpa(Nx=128, Nr=32, M=2, seed=14)
    cfg["laser_in"]["astig"] = 0.2
    sol, e, i, loop = build_product(cfg)
    osol, oe, oi, oloop = build_oracle(cfg)
    dens = cfg["eons_in"]["dens"]
    assert float(sol.DataDev["Ez_m2"].abs().max()) > 0
    assert compare_fields(sol, osol, dens=dens) < 1e-12
    loop.step()
    oloop.step()
    torch.cuda.synchronize()
    _sort_equal(e, oe)
    _sort_equal(i, oi)
    worst = compare_fields(sol, osol, dens=dens)
    assert worst < 1e-12, worst
    _particles_equal(e, oe, tol=1e-12)
