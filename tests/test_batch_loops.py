"""PIC_batch driving real PIC_loop objects on the CPU (fake solvers,
species and frames, fakes for torch's graph and stream objects, as in the
loop's own graph tests): in one-graph mode the first steps run each loop
alone, then one capture holds every loop's three pieces and later steps
are single replays, a window shift steps the loops through their own path
and the next step captures again; in streams mode each loop replays its
own three graphs."""
import contextlib

import pytest
import torch

import chimeracl_gb300.pic_loop as pl
from chimeracl_gb300.batch import PIC_batch
from tests.test_loop_graphs import FakeGraph, FakeStream, Frame, Solver, Species


@pytest.fixture
def loops(monkeypatch):
    log = []
    FakeGraph.log = log
    monkeypatch.setattr(torch.cuda, "CUDAGraph", FakeGraph)
    monkeypatch.setattr(torch.cuda, "Stream", FakeStream)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a: FakeStream())
    monkeypatch.setattr(torch.cuda, "stream", lambda s: contextlib.nullcontext())
    monkeypatch.setattr(pl.torch.cuda, "CUDAGraph", FakeGraph)
    import chimeracl_gb300._lib as lib
    monkeypatch.setattr(lib, "launch_count", lambda: len(log))
    out = []
    for _ in range(3):
        sol, sp = Solver(log), Species(log)
        out.append(pl.PIC_loop([sol], [sp], [Frame(sol, sp)], graphs=True))
    return out, log


def _step(b, log):
    del log[:]
    b.step()
    return list(log)


def test_one_graph_batch_with_real_loops(loops):
    lps, log = loops
    b = PIC_batch(lps, lanes=3, one_graph=True)
    b._sync = lambda: None
    s0 = _step(b, log)  # it = 0: each loop alone, eagerly (window shift)
    assert "capture_begin" not in s0 and s0.count("push_fields") == 3
    s1 = _step(b, log)  # it = 1: one capture of all loops' pieces, one replay
    assert s1.count("capture_begin") == 1 and s1.count("capture_end") == 1
    i0, i1 = s1.index("capture_begin"), s1.index("capture_end")
    assert s1[:i0].count("_phase") == 6  # 3 solvers x 2 directions, outside
    inside = s1[i0 + 1:i1]
    assert inside.count("push_fields") == 3 and inside.count("gather_and_push") == 3
    assert inside.count("sp.push_coords") == 6  # two half pushes per loop
    replays = [e for e in s1 if isinstance(e, tuple)]
    assert len(replays) == 1 and b.graph_captures == 1
    assert all(lp.it == 2 for lp in lps) and all(lp._graphs == {} for lp in lps)
    for _ in range(3):  # it = 2..4: one replay of the batch graph, nothing else
        assert _step(b, log) == replays
    s5 = _step(b, log)  # it = 5: window shift, each loop through its own step
    assert "capture_begin" in s5 and s5.count("push_fields") == 3
    assert b.graph_captures == 1
    s6 = _step(b, log)  # new signatures: the batch is captured again
    assert s6.count("capture_begin") == 1 and b.graph_captures == 2
    assert all(lp.it == 7 for lp in lps) and b.graph_replays == 5


def test_streams_batch_with_real_loops(loops):
    lps, log = loops
    b = PIC_batch(lps, lanes=2)
    for _ in range(2):  # it = 0 eager, it = 1 each loop captures its pieces
        _step(b, log)
    assert sum(lp.graph_captures for lp in lps) == 9
    s = _step(b, log)  # it = 2: each loop replays its own three graphs
    assert len(s) == 9 and all(isinstance(e, tuple) and e[0] == "replay" for e in s)
    assert all(lp.it == 3 for lp in lps)
