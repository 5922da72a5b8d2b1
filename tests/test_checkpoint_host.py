"""Step checkpoints on the CPU, with a stand-in loop whose step does what a
PIC step does to its state -- updates fields in place, exchanges buffers,
rebinds particle arrays on injection, draws from the injector's generator,
shifts host coordinate arrays in place, leaves lazily read device scalars
-- on CPU tensors: a run restored to a checkpoint and stepped again
reproduces the first run bit for bit; checkpoints survive a host round trip;
the recompute helper restores the last checkpoint before the asked step."""
import numpy as np
import pytest
import torch

from chimeracl_gb300.checkpoint import (Checkpointer, load_state_dict, restore_checkpoint,
                                        save_checkpoint, state_dict)
from chimeracl_gb300.methods.generic_methods_cu import ArgsDict, LazyScalar


class Obj:
    def __init__(self, seed, n):
        self.Args = ArgsDict(Np=n, Xgrid=np.linspace(-4.0, 0.0, 9), Xmin=-4.0)
        self.DataDev = {"x": torch.linspace(-4, 0, n, dtype=torch.float64),
                        "E": torch.zeros(5, dtype=torch.float64),
                        "dN0": torch.zeros(3), "dN1": torch.ones(3),
                        "_scratch": torch.zeros(2), "Np_stay_dev": torch.tensor([n])}
        self._rng = np.random.Generator(np.random.PCG64(seed))
        self.flag_sorted = False


class Loop:
    def __init__(self):
        self.solvers = [Obj(1, 0)]
        self.species = [Obj(2, 6), Obj(3, 6)]
        self.it = 0
        self._graphs = {"pa": object()}

    def step(self):
        sol = self.solvers[0]
        sol.DataDev["E"] += torch.from_numpy(sol._rng.random(5))  # in place
        sol.DataDev["dN0"], sol.DataDev["dN1"] = sol.DataDev["dN1"], sol.DataDev["dN0"]
        sol.DataDev["dN1"].mul_(2.0)
        for sp in self.species:
            D, A = sp.DataDev, sp.Args
            D["x"] += 0.1 * sol.DataDev["E"][0]
            D["_scratch"].fill_(float(self.it))  # scratch: rewritten every step
            if self.it % 3 == 0:  # a window shift: injection, host arrays moved
                new = torch.from_numpy(sp._rng.random(2))
                D["x"] = torch.cat([D["x"], new])
                A["Np"] = A["Np"] + 2
                A["Xgrid"] += 0.5  # in place, as Frame.shift_grids does
                D["Np_stay_dev"] = torch.tensor([A["Np"] - 1])
                dict.__setitem__(A, "Np_stay", LazyScalar(D["Np_stay_dev"]))
                dict.__setitem__(A, "right_lim", LazyScalar(D["x"].max(), cast=float))
                sp.flag_sorted = not sp.flag_sorted
        self.it += 1


def snapshot(loop):
    out = {}
    for kind, objs in (("sol", loop.solvers), ("sp", loop.species)):
        for i, o in enumerate(objs):
            for k, v in o.DataDev.items():
                if not k.startswith("_"):
                    out[(kind, i, k)] = v.clone()
            for k in o.Args:
                out[(kind, i, "arg:" + k)] = np.array(o.Args[k], copy=True)
            out[(kind, i, "rng")] = o._rng.random()  # advances: compare last
            out[(kind, i, "flag")] = o.flag_sorted
    out["it"] = loop.it
    return out


def assert_same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        if isinstance(a[k], torch.Tensor):
            assert torch.equal(a[k], b[k]), k
        else:
            np.testing.assert_array_equal(a[k], b[k], err_msg=str(k))


def test_restore_and_recompute_reproduce_the_run():
    loop = Loop()
    for _ in range(4):
        loop.step()
    ck = save_checkpoint(loop)
    assert ck.it == 4 and ck.nbytes() > 0
    assert "_scratch" not in ck.objs[("species", 0)]["dev"]
    for _ in range(6):
        loop.step()
    first = snapshot(loop)
    for _ in range(2):  # restorable more than once
        E, graphs = loop.solvers[0].DataDev["E"], loop._graphs
        loop._eager_left = 2  # as if a window shift had just been stepped
        restore_checkpoint(loop, ck)
        assert loop._eager_left == 0  # no eager steps pending after a restore
        # same-shape buffers restored in place: captured launches stay valid
        assert loop.it == 4 and loop.solvers[0].DataDev["E"] is E and loop._graphs is graphs
        for _ in range(6):
            loop.step()
        assert_same(first, snapshot(loop))


def test_checkpoint_state_dict_round_trip():
    import io
    loop = Loop()
    src = loop.species[0]
    loop.species[1].Args["InjectorSource"] = src  # a link, not a value
    for _ in range(5):
        loop.step()
    buf = io.BytesIO()
    torch.save(state_dict(save_checkpoint(loop)), buf)
    buf.seek(0)
    sd = torch.load(buf, weights_only=False)
    for _ in range(5):
        loop.step()
    first = snapshot(loop)
    restore_checkpoint(loop, load_state_dict(sd, "cpu"))
    assert loop.species[1].Args["InjectorSource"] is src
    for _ in range(5):
        loop.step()
    assert_same(first, snapshot(loop))


def test_checkpointer_recompute():
    loop = Loop()
    ref = Loop()
    cp = Checkpointer(loop, every=4)
    cp.run(11)
    assert sorted(cp.checkpoints) == [0, 4, 8]
    for _ in range(7):
        ref.step()
    assert cp.recompute(7) == 7
    assert_same(snapshot(ref), snapshot(loop))
    with pytest.raises(ValueError):
        Checkpointer(loop, every=0)
