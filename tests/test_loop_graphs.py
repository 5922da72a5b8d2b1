"""PIC_loop's graph bookkeeping on the CPU, with fakes for torch's CUDA graph
and stream objects and stub solver / species / frame objects: which pieces
are captured, replayed or run eagerly, step by step, and what forces a
capture."""
import contextlib

import pytest
import torch

import chimeracl_gb300.pic_loop as pl


class FakeGraph:
    log = None

    def capture_begin(self):
        FakeGraph.log.append("capture_begin")

    def capture_end(self):
        FakeGraph.log.append("capture_end")

    def replay(self):
        FakeGraph.log.append(("replay", id(self)))


class FakeStream:
    def wait_stream(self, other):
        pass


class Solver:
    def __init__(self, log):
        self.log = log
        self.Args = {"M": 0, "Xmin": 0.0, "vec_comps": ["x", "y", "z"]}
        self.DataDev = {"E": torch.zeros(4), "rho": torch.zeros(4)}
        for c in "xyz":
            self.DataDev["dN0" + c + "_fb_m0"] = torch.zeros(2)
            self.DataDev["dN1" + c + "_fb_m0"] = torch.ones(2)

    def __getattr__(self, name):  # every solver method: log the call
        if name.startswith("__"):
            raise AttributeError(name)
        return lambda *a, **k: self.log.append(name)

    def _real_dev(self, name):
        return torch.zeros(1)


class Species:
    def __init__(self, log):
        self.log = log
        self.Args = {"Np": 10}
        self.DataDev = {"x": torch.zeros(10)}

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return lambda *a, **k: self.log.append("sp." + name)


class Frame:
    def __init__(self, solver, species, steps=5):
        self.Args = {"Steps": steps}
        self.sol, self.sp = solver, species

    def shift_grids(self, grids):
        self.sol.Args["Xmin"] += 1.0

    def inject_plasma(self, species, grid):
        self.sp.DataDev["x"] = torch.zeros(12)  # new arrays, new count
        self.sp.Args["Np"] = 12


@pytest.fixture
def loop(monkeypatch):
    log = []
    FakeGraph.log = log
    monkeypatch.setattr(torch.cuda, "CUDAGraph", FakeGraph)
    monkeypatch.setattr(torch.cuda, "Stream", FakeStream)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a: FakeStream())
    monkeypatch.setattr(torch.cuda, "stream", lambda s: contextlib.nullcontext())
    monkeypatch.setattr(pl.torch.cuda, "CUDAGraph", FakeGraph)
    import chimeracl_gb300._lib as lib
    monkeypatch.setattr(lib, "launch_count", lambda: len(log))
    sol, sp = Solver(log), Species(log)
    lp = pl.PIC_loop([sol], [sp], [Frame(sol, sp)], graphs=True)
    return lp, log, sol, sp


def _step(lp, log):
    del log[:]
    lp.step()
    return list(log)


def test_pieces_captured_replayed_and_kept_through_shifts(loop):
    lp, log, sol, sp = loop
    first = _step(lp, log)  # it = 0: eager, window shift included
    assert "capture_begin" not in first and not any(isinstance(e, tuple) for e in first)
    assert "push_fields" in first and "sp.push_coords" in first
    s1 = _step(lp, log)  # it = 1: the three pieces captured, then replayed
    assert s1.count("capture_begin") == 3 and sum(isinstance(e, tuple) for e in s1) == 3
    objs = {p: g[0] for p, g in lp._graphs.items()}  # held: their ids stay unique
    ids = {p: id(g) for p, g in objs.items()}
    # phases refreshed before the field piece's capture, not inside it
    cap_f = [i for i, e in enumerate(s1) if e == "capture_begin"][1]
    assert s1[cap_f - 2:cap_f] == ["_phase", "_phase"]
    for _ in range(3):  # it = 2..4: replays only, no library call from Python
        s = _step(lp, log)
        assert s == [("replay", ids["pa"]), ("replay", ids["f"]), ("replay", ids["pb"])]
    s5 = _step(lp, log)  # it = 5: window shift, the particle pieces eager
    assert s5.count("capture_begin") == 0
    assert ("replay", ids["f"]) in s5  # the field solve replays through the shift
    assert "push_fields" not in s5  # ... and is not run eagerly
    assert s5.index("sp.push_coords") < s5.index(("replay", ids["f"])) < s5.index("gather_and_push")
    assert lp.eager_after_shift == 2
    for _ in range(lp.eager_after_shift):  # it = 6, 7: still eager (host gets ahead)
        s = _step(lp, log)
        assert s.count("capture_begin") == 0 and "sp.push_coords" in s
        assert ("replay", ids["f"]) in s
    s8 = _step(lp, log)  # it = 8: the particle pieces captured again, then replayed
    assert s8.count("capture_begin") == 2
    assert lp._graphs["f"][0] is objs["f"] and lp._graphs["pa"][0] is not objs["pa"]
    s9 = _step(lp, log)
    assert s9.count("capture_begin") == 0 and len(s9) == 3
    assert lp.graph_replays == 9 and lp.graph_captures == 5


def test_capture_at_the_shift_when_no_eager_steps(loop):
    lp, log, sol, sp = loop
    lp.eager_after_shift = 0  # what a batch of runs uses
    for _ in range(5):
        _step(lp, log)
    f_graph = lp._graphs["f"][0]
    s5 = _step(lp, log)  # it = 5: shift; pieces eager, then captured right away
    assert s5.count("capture_begin") == 2
    assert s5.index("sp.push_coords") < s5.index("capture_begin")
    assert lp._graphs["f"][0] is f_graph
    s6 = _step(lp, log)
    assert s6.count("capture_begin") == 0 and len(s6) == 3


def test_rebound_buffers_force_a_capture(loop):
    lp, log, sol, sp = loop
    lp.eager_after_shift = 0  # the step at it = 5 (a shift) captures at once
    for _ in range(3):
        _step(lp, log)
    sol.DataDev["E"] = torch.zeros(4)  # a solver buffer rebound: all pieces
    s = _step(lp, log)
    assert s.count("capture_begin") == 3
    sp.DataDev["x"] = torch.zeros(10)  # a particle array rebound: particle pieces
    s = _step(lp, log)
    assert s.count("capture_begin") == 2
    sp.Args["Np"] = 9  # a new count: particle pieces
    s = _step(lp, log)
    assert s.count("capture_begin") == 2
    sol.DataDev["phs_shft"] = torch.zeros(1)  # the phase alias is not part of it
    s = _step(lp, log)
    assert s.count("capture_begin") == 0


def test_graphs_off_or_diagnostics_run_eagerly(loop):
    lp, log, sol, sp = loop
    lp.graphs = False
    for _ in range(3):
        s = _step(lp, log)
        assert "capture_begin" not in s and "push_fields" in s

    class Diag:
        def make_record(self, it):
            log.append(("record", it))

    lp.graphs, lp.diags = True, [Diag()]
    s = _step(lp, log)
    assert s[0] == ("record", 3) and "capture_begin" not in s and "push_fields" in s
