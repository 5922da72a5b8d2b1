"""PIC_batch's scheduling on the CPU, with fakes for torch's stream objects
and for the runs: every run stepped once per batch step on a stream of its
own, the lane chaining (run i after run i - lanes), one lane while any run
takes its first step, and the lane autotuner (the fastest candidate kept;
window-shift and capturing steps left out of its timings)."""
import contextlib

import pytest
import torch

import chimeracl_gb300.batch as bm


class FakeStream:
    log = None
    count = 0

    def __init__(self, name=None):
        FakeStream.count += 1
        self.name = name if name is not None else "s%d" % (FakeStream.count - 1)

    def wait_stream(self, other):
        FakeStream.log.append(("wait", self.name, other.name))


class FakeLoop:
    def __init__(self, idx, log, steps=5, capture_at=()):
        self.idx, self.log = idx, log
        self.it = 0
        self.graphs, self.timit, self.diags = True, False, []
        self.graph_captures = 0
        self.frame_steps = steps
        self.capture_at = set(capture_at)
        self.species = []

    def _frame_due(self):
        return self.it % self.frame_steps == 0

    def step(self):
        self.log.append(("step", self.idx, bm.torch.cuda.current_stream().name))
        if self.it in self.capture_at:
            self.graph_captures += 1
        self.it += 1


@pytest.fixture
def fakes(monkeypatch):
    log = []
    FakeStream.log, FakeStream.count = log, 0
    default = FakeStream("cur")
    FakeStream.count = 0
    state = {"cur": default}

    @contextlib.contextmanager
    def use(s):
        prev, state["cur"] = state["cur"], s
        try:
            yield
        finally:
            state["cur"] = prev

    monkeypatch.setattr(torch.cuda, "Stream", FakeStream)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a: state["cur"])
    monkeypatch.setattr(torch.cuda, "stream", use)
    return log


def test_lane_of_deals_runs_round_robin():
    assert bm.PIC_batch.lane_of(5, 2) == [[0, 2, 4], [1, 3]]
    assert bm.PIC_batch.lane_of(3, 3) == [[0], [1], [2]]
    assert bm.PIC_batch.lane_of(4, 1) == [[0, 1, 2, 3]]


def test_arguments_checked():
    with pytest.raises(ValueError):
        bm.PIC_batch([])
    with pytest.raises(ValueError):
        bm.PIC_batch([object()] * 3, lanes=4)
    with pytest.raises(ValueError):
        bm.PIC_batch([object()] * 3, candidates=(5, 8))


def test_each_run_on_its_own_stream_chained_by_lanes(fakes):
    log = fakes
    loops = [FakeLoop(i, log) for i in range(5)]
    b = bm.PIC_batch(loops, lanes=2)
    b.step()  # first steps: one lane whatever `lanes` says
    waits = [e for e in log if e[0] == "wait" and e[1] != "cur"]
    assert waits == [("wait", "s0", "cur"), ("wait", "s1", "s0"), ("wait", "s2", "s1"),
                     ("wait", "s3", "s2"), ("wait", "s4", "s3")]
    log.clear()
    b.step()
    steps = [e for e in log if e[0] == "step"]
    assert steps == [("step", i, "s%d" % i) for i in range(5)]  # streams kept
    waits = [e for e in log if e[0] == "wait" and e[1] != "cur"]
    assert waits == [("wait", "s0", "cur"), ("wait", "s1", "cur"), ("wait", "s2", "s0"),
                     ("wait", "s3", "s1"), ("wait", "s4", "s2")]
    joins = [e for e in log if e[0] == "wait" and e[1] == "cur"]
    assert joins == [("wait", "cur", "s%d" % i) for i in range(5)]
    assert all(lp.it == 2 for lp in loops) and b.it == 2


def test_autotuner_keeps_the_fastest_lane_count(fakes):
    log = fakes
    loops = [FakeLoop(i, log, steps=7, capture_at=(1, 8)) for i in range(4)]
    b = bm.PIC_batch(loops, candidates=(1, 2, 4), tune_steps=2)
    t = [0.0]
    cost = {1: 3.0, 2: 1.0, 4: 2.0}
    issued = []
    orig = b._issue

    def issue(k):
        issued.append(k)
        t[0] += cost[k]
        orig(k)

    b._issue, b._clock, b._sync = issue, (lambda: t[0]), (lambda: None)
    b.run(16)
    # step 0: first steps (one lane); step 7 shifts the window (untimed, all
    # lanes); steps 1 and 8 capture (timed, discarded).  Timed steps go to
    # the candidates in order.
    assert issued[:3] == [1, 1, 1] and issued[7] == 4
    assert {c: len(v) for c, v in b.tune_log.items()} == {1: 2, 2: 2, 4: 2}
    assert all(v == [cost[c]] * 2 for c, v in b.tune_log.items())
    assert b.lanes == 2
    assert issued[-3:] == [2, 2, 2]
    assert all(lp.it == 16 for lp in loops)


def test_runs_that_never_replay_keep_all_lanes(fakes):
    log = fakes
    loops = [FakeLoop(i, log) for i in range(3)]
    for lp in loops:
        lp.diags = ["a diagnostic"]  # eager steps: never timed
    b = bm.PIC_batch(loops, candidates=(1, 3))
    b._sync = lambda: None
    b.run(6)
    assert b.lanes is None and all(len(v) == 0 for v in b.tune_log.values())
    log.clear()
    b.step()
    waits = [e for e in log if e[0] == "wait" and e[1] != "cur"]
    assert waits == [("wait", "s%d" % i, "cur") for i in range(3)]


class FakeGraph:
    log = None

    def capture_begin(self):
        FakeGraph.log.append(("capture_begin",))

    def capture_end(self):
        FakeGraph.log.append(("capture_end",))

    def replay(self):
        FakeGraph.log.append(("replay", id(self)))


class FakeSolver:
    def __init__(self, log, idx):
        self.log, self.idx = log, idx

    def _phase(self, d):
        self.log.append(("phase", self.idx, d))


class PieceLoop(FakeLoop):
    """A run whose step pieces log the stream they are issued on; its
    signature changes at each window shift (new origin)."""

    def __init__(self, idx, log, steps=5):
        super().__init__(idx, log, steps=steps)
        self.solvers = [FakeSolver(log, idx)]
        self.graph_replays = 0
        self.origin = 0

    def _signature(self, piece):
        return (self.idx, self.origin), ()

    def step(self):
        if self._frame_due():
            self.origin += 1
        super().step()

    def _piece(self, name):
        self.log.append((name, self.idx, bm.torch.cuda.current_stream().name))

    def _particles_before(self, graph_mode):
        assert graph_mode
        self._piece("pa")

    def _fields(self, graph_mode):
        self._piece("f")

    def _particles_after(self, graph_mode):
        self._piece("pb")


def test_one_graph_captures_once_and_replays(fakes, monkeypatch):
    log = fakes
    FakeGraph.log = log
    monkeypatch.setattr(torch.cuda, "CUDAGraph", FakeGraph)
    from chimeracl_gb300 import _lib
    monkeypatch.setattr(_lib, "launch_count", lambda: 0)
    loops = [PieceLoop(i, log, steps=5) for i in range(3)]
    b = bm.PIC_batch(loops, lanes=2, one_graph=True)
    b.step()  # first steps: each run alone
    assert b.graph_captures == 0 and all(lp.it == 1 for lp in loops)
    log.clear()
    b.step()  # captured, then replayed once
    i0 = log.index(("capture_begin",))
    i1 = log.index(("capture_end",))
    # phases refreshed before the capture, outside it
    assert all(("phase", i, d) in log[:i0] for i in range(3) for d in (0, 1))
    inside = log[i0 + 1:i1]
    pieces = [e for e in inside if e[0] in ("pa", "f", "pb")]
    assert pieces == [(p, i, "s%d" % i) for i in range(3) for p in ("pa", "f", "pb")]
    forks = [e for e in inside if e[0] == "wait" and e[1] != "s3"]
    # s3 is the capture stream: runs 0, 1 fork from it, run 2 from run 0
    assert forks == [("wait", "s0", "s3"), ("wait", "s1", "s3"), ("wait", "s2", "s0")]
    joins = [e for e in inside if e[0] == "wait" and e[1] == "s3"]
    assert joins == [("wait", "s3", "s%d" % i) for i in range(3)]
    assert [e[0] for e in log[i1:]].count("replay") == 1
    assert b.graph_captures == 1 and b.graph_replays == 1 and all(lp.it == 2 for lp in loops)
    log.clear()
    b.run(2)  # steps 2, 3: replays only
    assert not any(e[0] in ("capture_begin", "pa") for e in log)
    assert [e[0] for e in log].count("replay") == 2 and b.graph_captures == 1
    log.clear()
    b.step()  # step 4: no shift yet (it = 4); replay
    b.step()  # step 5: window shift, every run alone
    assert [e[0] for e in log].count("replay") == 1
    assert all(lp.origin == 2 for lp in loops)
    b.step()  # new signatures: captured again
    assert b.graph_captures == 2 and all(lp.it == 7 for lp in loops)


def test_batch_runs_capture_at_their_window_shift(fakes):
    """A batch keeps the host busy with all its runs' launches: its loops
    capture their particle pieces right at a window shift (no eager steps
    after it), and a run with eager steps pending makes a batch step
    ineligible for one graph / autotuning."""
    log = fakes
    loops = [FakeLoop(i, log) for i in range(3)]
    for lp in loops:
        lp.eager_after_shift, lp._eager_left = 2, 0
    b = bm.PIC_batch(loops, lanes=1)
    assert all(lp.eager_after_shift == 0 for lp in loops)
    for lp in loops:
        lp.it = 3
    assert b._eligible()
    loops[1]._eager_left = 1
    assert not b._eligible()
