"""The mixed-precision form (FP32 particles and fields, BF16x3 tensor-core
Hankel GEMMs) against the FP64 oracle on the same seeded LPA run: integrated
diagnostics -- field energy, on-axis Ez wake amplitude -- within 1e-4
relative after 40 steps (two window shifts), the bar the mixed form is held
to; kinetic energy reported."""
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


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_reduced_precision_vs_fp64_oracle(cuda, precision):
    cfg = small_lpa(Nx=256, Nr=32, M=1, seed=17)
    sol, e, i, loop = build_product(cfg, precision=precision)
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
    assert err["kinetic"] < 1e-2, err
