"""The mixed-precision form (FP32 particles and fields, BF16x3 tensor-core
Hankel GEMMs) against the FP64 oracle on the same seeded LPA run: integrated
diagnostics -- field energy, the wake (max |Ex_m0| on the axis: x is the
propagation axis in these arrays) and the laser's on-axis amplitude (max
|Ez_m0|) -- within 1e-4 relative after 40 steps (two window shifts), the bar
the mixed form is held to; kinetic energy within 1e-2."""
import numpy as np
import pytest
import torch

from oracle import pic_oracle as po
from tests.lpa_setup import build_oracle, build_product, small_lpa

pytestmark = pytest.mark.gpu


def product_diagnostics(sol, eons):
    A, D = sol.Args, sol.DataDev

    class O:  # view in the oracle's layout
        pass
    o = O()
    o.Args = A
    o.D = {k: D[k].detach().cpu().numpy().astype(np.complex128 if D[k].is_complex() else np.float64)
           for k in D if k[0] in "EB" and "_fb" not in k}
    p = O()
    p.Args = {"Np": eons.Args["Np"]}
    p.D = {"w": eons.DataDev["w"].double().cpu().numpy(),
           "g_inv": eons.DataDev["g_inv"].double().cpu().numpy()}
    return po.diagnostics(o, [p])


@pytest.mark.parametrize("precision,comp", [("mixed", False), ("fp32", False), ("mixed", True)])
def test_reduced_precision_vs_fp64_oracle(cuda, precision, comp):
    cfg = small_lpa(Nx=256, Nr=32, M=1, seed=17)
    sol, e, i, loop = build_product(cfg, precision=precision, compensated_positions=comp)
    osol, oe, oi, oloop = build_oracle(cfg)
    for _ in range(40):
        loop.step()
        oloop.step()
    torch.cuda.synchronize()
    got = product_diagnostics(sol, e)
    ref = po.diagnostics(osol, [oe, oi])
    err = {k: abs(got[k] / ref[k] - 1) for k in ref}
    assert err["field_energy"] < 1e-4, err
    assert err["ez_axis_max"] < 1e-4, err
    assert err["wake_ex_max"] < 1e-4, err
    assert err["kinetic"] < 1e-2, err


def test_compensated_positions_through_window_shifts(cuda):
    """The low parts travel with their particles through injection, sort and
    align: after three window shifts every mobile particle has them, each
    within half a unit in the last place of its coordinate, and the
    coordinates stay close to those of the plain FP32 run."""
    cfg = small_lpa(Nx=256, Nr=32, M=1, seed=5)
    runs = {c: build_product(cfg, precision="mixed", compensated_positions=c)
            for c in (False, True)}
    for _ in range(61):
        for r in runs.values():
            r[3].step()
    torch.cuda.synchronize()
    e = runs[True][1]
    D = e.DataDev
    # immobile ions carry low parts too (their charge sits on the electrons')
    assert "x_lo" in D and "x_lo" in runs[True][2].DataDev
    for c in ("x", "y", "z"):
        hi, lo = D[c].cpu().numpy(), D[c + "_lo"].cpu().numpy()
        assert hi.shape == lo.shape == (e.Args["Np"],)
        assert np.all(np.abs(lo) <= 0.5 * np.spacing(np.abs(hi)))
        assert np.count_nonzero(lo) > lo.size // 4
    e0 = runs[False][1]
    assert e0.Args["Np"] == e.Args["Np"]
    # (sorted: a particle that crossed a cell face in one run only shifts
    # the cell order of the arrays)
    diff = np.abs(np.sort(D["x"].cpu().numpy()) - np.sort(e0.DataDev["x"].cpu().numpy()))
    assert np.median(diff) < 1e-2 * runs[True][0].Args["dx"]
