"""Step checkpoints on the GPU: a run (FP64 and mixed forms, CUDA graphs on)
restored to a checkpoint taken between window shifts and stepped on through
the next shift gives, bit for bit, the fields, particles and counts of the
first pass; so does the same checkpoint after a round trip through host
memory."""
import pytest
import torch

from chimeracl_gb300.checkpoint import (load_state_dict, restore_checkpoint, save_checkpoint,
                                        state_dict)
from tests.lpa_setup import build_product, small_lpa

pytestmark = pytest.mark.gpu


def _state(sol, eons, ions):
    st = {("sol", k): v.clone() for k, v in sol.DataDev.items()
          if isinstance(v, torch.Tensor) and not k.startswith(("_", "buff_fb", "phs", "fld_buff"))}
    for tag, sp in (("e", eons), ("i", ions)):
        for k in ("x", "y", "z", "w") + (("px", "py", "pz", "g_inv") if tag == "e" else ()):
            st[(tag, k)] = sp.DataDev[k].clone()
        st[(tag, "Np")] = sp.Args["Np"]
    return st


def _assert_same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        if isinstance(a[k], torch.Tensor):
            assert torch.equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restored_run_reproduces_the_first_pass(cuda, precision):
    cfg = small_lpa(Nx=128, Nr=32, M=1, seed=29, steps=10)
    sol, eons, ions, loop = build_product(cfg, precision=precision)
    loop.graphs = True
    for _ in range(13):
        loop.step()
    ck = save_checkpoint(loop)
    for _ in range(12):  # through the window shift at step 20
        loop.step()
    torch.cuda.synchronize()
    first = _state(sol, eons, ions)
    for ckpt in (ck, load_state_dict(state_dict(ck), cuda)):
        restore_checkpoint(loop, ckpt)
        assert loop.it == 13
        for _ in range(12):
            loop.step()
        torch.cuda.synchronize()
        _assert_same(first, _state(sol, eons, ions))
