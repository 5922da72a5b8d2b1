"""PIC_batch on the GPU: three mixed-precision runs of uneven grid sizes
(256 x 32, 128 x 32, 64 x 24; different seeds, densities and lasers),
stepped together through two window shifts with the lane autotuner active
-- each run's step on its own stream, or the whole batch step as one CUDA
graph -- give bit for bit the fields and particles of the same runs stepped
one after the other on one stream."""
import pytest
import torch

from chimeracl_gb300.batch import PIC_batch
from tests.lpa_setup import build_product, small_lpa

pytestmark = pytest.mark.gpu

CASES = [dict(Nx=256, Nr=32, seed=41, a0=2.0, dens=1e-3, R=6.0),
         dict(Nx=128, Nr=32, seed=42, a0=1.5, dens=2e-3, R=5.0),
         dict(Nx=64, Nr=24, seed=43, a0=2.5, dens=5e-4, R=4.0)]
STEPS = 25


def _runs():
    runs = []
    for c in CASES:
        cfg = small_lpa(M=1, nppc=(1, 1, 4), steps=10, **c)
        sol, e, i, loop = build_product(cfg, precision="mixed")
        loop.graphs = True
        runs.append((sol, e, i, loop))
    return runs


@pytest.fixture(scope="module")
def alone(cuda):
    runs = _runs()
    for r in runs:
        for _ in range(STEPS):
            r[3].step()
    torch.cuda.synchronize()
    return runs


def _assert_same(alone, batched):
    for (s0, e0, i0, _), (s1, e1, i1, _) in zip(alone, batched):
        for k, v in s0.DataDev.items():
            if isinstance(v, torch.Tensor) and not k.startswith(("_", "buff_fb", "phs",
                                                                 "fld_buff")):
                assert torch.equal(v, s1.DataDev[k]), k
        assert e0.Args["Np"] == e1.Args["Np"] and i0.Args["Np"] == i1.Args["Np"]
        for k in ("x", "y", "z", "px", "py", "pz", "g_inv", "w"):
            assert torch.equal(e0.DataDev[k], e1.DataDev[k]), k
        for k in ("x", "y", "z", "w"):
            assert torch.equal(i0.DataDev[k], i1.DataDev[k]), k


def test_batched_runs_equal_runs_stepped_alone(alone):
    batched = _runs()
    torch.cuda.synchronize()
    b = PIC_batch([r[3] for r in batched], candidates=(1, 2, 3), tune_steps=2)
    b.run(STEPS)
    torch.cuda.synchronize()
    assert {c: len(v) for c, v in b.tune_log.items()} == {1: 2, 2: 2, 3: 2}
    assert b.lanes in (1, 2, 3)
    assert all(r[3].it == STEPS for r in batched)
    assert all(r[3].graph_replays >= STEPS - 1 for r in batched)
    _assert_same(alone, batched)


def test_one_graph_batch_equals_runs_stepped_alone(alone):
    batched = _runs()
    torch.cuda.synchronize()
    b = PIC_batch([r[3] for r in batched], candidates=(1, 3), tune_steps=2, one_graph=True)
    b.run(STEPS)
    torch.cuda.synchronize()
    assert {c: len(v) for c, v in b.tune_log.items()} == {1: 2, 3: 2}
    # steps 1-9, 11-19, 21-24 are batch replays; every shift forces a capture
    assert b.graph_replays == STEPS - 3 and b.graph_captures >= 3
    assert all(r[3].it == STEPS for r in batched)
    _assert_same(alone, batched)
