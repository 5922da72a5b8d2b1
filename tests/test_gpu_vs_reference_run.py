"""The product against a committed run of the reference's own kernels: the
1024 x 128, M = 1 grid on the 512 x 64 run's window (2x2x4 per cell, a0 = 2
laser, window shift with injection at the first step) for 20 FP64 steps
through the public API -- the same particle counts, and field energy,
on-axis Ez amplitude and kinetic energy within 1e-8 relative of the
reference kernels' run (tests/golden/lpa_m1_1024x128_20steps.npz)."""
import os

import numpy as np
import pytest
import torch

from oracle.pic_oracle import diagnostics
from tests.lpa_setup import build_product, to_np

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                      "lpa_m1_1024x128_20steps.npz")


class _Host:
    def __init__(self, obj):
        self.Args = obj.Args
        self.D = {k: to_np(v) for k, v in obj.DataDev.items() if isinstance(v, torch.Tensor)}


def test_fp64_run_matches_reference_kernels_run(cuda):
    from tests.golden.make_golden import golden_run
    case, cfg = golden_run("lpa_m1_1024x128_20steps.npz")
    g = np.load(GOLDEN)
    sol, eons, ions, loop = build_product(cfg, precision="fp64")
    for _ in range(case["nsteps"]):
        loop.step()
    torch.cuda.synchronize()
    assert eons.Args["Np"] == int(g["count:Np"])
    got = diagnostics(_Host(sol), [_Host(eons)])
    for k, v in got.items():
        ref = float(g["diag:" + k])
        assert abs(v / ref - 1.0) < 1e-8, (k, v, ref)
