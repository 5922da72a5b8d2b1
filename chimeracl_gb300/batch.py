"""Many independent runs on one GPU, stepped together.

The reference runs one simulation per process (``PIC_loop.step()``,
chimeraCL/pic_loop.py:57-142).  Small grids leave most of a GB300 idle: a
256 x 32 run's step is ~100 short kernels, each filling a few of the 152
SMs, and the host's launch rate bounds it.  ``PIC_batch`` steps many such
runs (uneven grid sizes, densities, lasers) side by side: every run keeps
its own ``PIC_loop`` (with ``graphs=True`` its step is three CUDA-graph
replays) and is issued on a CUDA stream of its own, so that the runs'
kernels execute concurrently and the device, not the host, is the bound.

Each run's kernels keep their order on its stream, and no kernel of a step
reads another run's buffers, so a batched run's results are bitwise those
of the same run stepped alone (the kernels are deterministic: no atomics in
the deposits, a stable sort, fixed reduction orders).  A run stays on its
own stream for its whole life, so every buffer it allocates, uses and frees
belongs to that stream's allocator pool: no other run can be handed a block
while the run's kernels still read it.

Lanes.  ``lanes`` bounds how many runs execute at once: lane l runs l,
l + lanes, l + 2 lanes, ... one after the other (run i's stream waits for
run i - lanes' step), and the lanes run concurrently.  With ``lanes=None``
the batch picks the count itself while the runs advance: the first eligible
steps try each candidate in turn (``tune_steps`` timed steps each), the
smallest median host time per step (issue to device idle) wins, and later
steps use it.  A step is eligible when no run shifts its window and no run
captures a graph in it (those steps run eagerly and capture; their time
says nothing about the lane count); steps that are not run with the
largest candidate, so runs that never replay graphs (diagnostics attached,
timers on) keep full concurrency.  Results do not depend on the lane
count, so tuning on the real steps costs only the slower candidates' time.

First steps.  A run's first step builds the library's lazily created,
shared read-only tables (FFT twiddles per transform length) on its stream;
steps in which any run takes its first step therefore run as one lane, so
that every later use of a table is ordered after the launch that fills it.

Window shifts.  A run whose window shifts in a step reads two device
scalars on the host (``Np_stay``, ``right_lim``); those reads wait for that
run's stream only, while the other runs' kernels keep executing.

One graph (``one_graph=True``).  On an eligible step (below) the whole
batch step -- every run's particle work, field solve and gather + push, on
the runs' streams with the lane chaining -- is captured into one CUDA graph
on a capture stream that the runs' streams fork from and join back to, and
replayed with one launch per batch step while no run's signature changes
(its device buffers, particle counts, grid origin) and the lane count
stays.  A run's window shift steps it alone (eagerly, on its stream) and
changes its signature, so the next eligible step captures the batch again.
Each run's phase factors are refreshed before a capture, outside it.

CUDA maps streams onto ``CUDA_DEVICE_MAX_CONNECTIONS`` hardware queues (8
unless that variable is set before CUDA starts); lanes beyond that share
queues."""
import statistics
import time

import torch

from .pic_loop import capture_guard


class PIC_batch:
    def __init__(self, loops, lanes=None, candidates=None, tune_steps=3, one_graph=False):
        self.loops = list(loops)
        if not self.loops:
            raise ValueError("PIC_batch needs at least one run")
        n = len(self.loops)
        if lanes is not None:
            lanes = int(lanes)
            if not 1 <= lanes <= n:
                raise ValueError(f"lanes={lanes} outside [1, {n}]")
        self.lanes = lanes
        if candidates is None:
            candidates = (1, 2, 4, 8, 16, 32, 64, n)
        self.candidates = sorted({int(c) for c in candidates if 1 <= int(c) <= n})
        if not self.candidates:
            raise ValueError("no lane count among the candidates fits the batch")
        self.tune_steps = int(tune_steps)
        for lp in self.loops:
            # the batch keeps the host busy with many runs' launches: a run
            # captures its pieces again right at its window shift
            if hasattr(lp, "eager_after_shift"):
                lp.eager_after_shift = 0
        # candidate -> host seconds of its timed steps
        self.tune_log = {c: [] for c in self.candidates}
        self._streams = None
        self.one_graph = bool(one_graph)
        # [graph, signature, refs kept alive, library launches captured]
        self._bgraph = None
        self._cap_stream = None
        self.graph_captures = 0  # batch graphs captured
        self.graph_replays = 0  # batch steps served by one graph replay
        self.graph_kernels_captured = 0
        self.graph_kernels_replayed = 0
        self.it = 0
        # replaceable for tests: a clock and a device-wide synchronisation
        self._clock = time.perf_counter
        self._sync = torch.cuda.synchronize

    # -----------------------------------------------------------------
    @staticmethod
    def lane_of(nruns, lanes):
        """Run indices per lane, in execution order (lane l takes runs l,
        l + lanes, ...)."""
        return [list(range(l, nruns, lanes)) for l in range(lanes)]

    def _candidate(self):
        """The lane count still being timed, or None once tuning is done."""
        for c in self.candidates:
            if len(self.tune_log[c]) < self.tune_steps:
                return c
        return None

    def _pick(self):
        self.lanes = min(self.candidates, key=lambda c: statistics.median(self.tune_log[c]))
        return self.lanes

    def _eligible(self):
        """No window shift due in any run and every run past its first
        (eager) step: the step replays graphs only, unless a signature
        changed (checked after the step through the capture count)."""
        for lp in self.loops:
            if (lp.it == 0 or lp._frame_due() or lp.timit or lp.diags
                    or getattr(lp, "_eager_left", 0)):
                return False
            if not (lp.graphs or self.one_graph):
                return False
        return True

    # -----------------------------------------------------------------
    def _issue(self, k):
        """One step of every run: run i on its own stream, after the
        current stream's work (i < k) or after run i - k's step; the
        current stream then waits for every run."""
        cur = torch.cuda.current_stream()
        if self._streams is None:
            self._streams = [torch.cuda.Stream() for _ in self.loops]
        for i, (lp, s) in enumerate(zip(self.loops, self._streams)):
            s.wait_stream(cur if i < k else self._streams[i - k])
            with torch.cuda.stream(s):
                lp.step()
        for s in self._streams:
            cur.wait_stream(s)

    def _batch_signature(self, k):
        sigs = [lp._signature("pa") for lp in self.loops]
        return (k,) + tuple(sg[0] for sg in sigs), tuple(sg[1] for sg in sigs)

    def _capture_batch(self, k):
        """Capture one step of every run into one graph: run i on its own
        stream, forked from the capture stream (i < k) or from run i - k's
        stream, all joined back before the capture ends."""
        from . import _lib
        self._bgraph = None
        for lp in self.loops:
            for sol in lp.solvers:  # phase factors for the current origin
                sol._phase(0)
                sol._phase(1)
        if self._streams is None:
            self._streams = [torch.cuda.Stream() for _ in self.loops]
        if self._cap_stream is None:
            self._cap_stream = torch.cuda.Stream()
        cap, streams = self._cap_stream, self._streams
        n0 = _lib.launch_count()
        g = torch.cuda.CUDAGraph()
        cur = torch.cuda.current_stream()
        cap.wait_stream(cur)
        with torch.cuda.stream(cap), capture_guard():
            g.capture_begin()
            try:
                for i, (lp, s) in enumerate(zip(self.loops, streams)):
                    s.wait_stream(cap if i < k else streams[i - k])
                    with torch.cuda.stream(s):
                        lp._particles_before(graph_mode=True)
                        lp._fields(graph_mode=True)
                        lp._particles_after(graph_mode=True)
                for s in streams:
                    cap.wait_stream(s)
            finally:
                g.capture_end()
        cur.wait_stream(cap)
        nk = _lib.launch_count() - n0
        sig, refs = self._batch_signature(k)
        self._bgraph = [g, sig, refs, nk]
        self.graph_captures += 1
        self.graph_kernels_captured += nk

    def _replay_batch(self, k):
        """One batch step as one graph replay (captured first when the
        signature changed)."""
        if self._bgraph is None or self._batch_signature(k)[0] != self._bgraph[1]:
            self._capture_batch(k)
        self._bgraph[0].replay()
        self.graph_kernels_replayed += self._bgraph[3]
        for lp in self.loops:
            lp.it += 1
            lp.graph_replays += 1
        self.graph_replays += 1

    def _run(self, k):
        if self.one_graph and self._eligible():
            self._replay_batch(k)
        else:
            self._issue(k)

    def _captures(self):
        return self.graph_captures + sum(lp.graph_captures for lp in self.loops)

    def step(self):
        cand = None
        if any(lp.it == 0 for lp in self.loops):
            k = 1  # first steps build shared tables: one lane
        elif self.lanes is not None:
            k = self.lanes
        else:
            cand = self._candidate()
            if cand is None:
                k = self._pick()
            elif self._eligible():
                k = cand
            else:
                # an untimed step while tuning (window shift, capture, or
                # runs that never replay graphs): all lanes
                k, cand = self.candidates[-1], None
        if cand is not None:
            caps0 = self._captures()
            self._sync()
            t0 = self._clock()
            self._run(k)
            self._sync()
            dt = self._clock() - t0
            if self._captures() == caps0:
                self.tune_log[cand].append(dt)
        else:
            self._run(k)
        self.it += 1
        return self.it

    def run(self, nsteps):
        for _ in range(int(nsteps)):
            self.step()
        return self.it

    def electrons(self):
        """Mobile electrons over all runs (each run's first species)."""
        return sum(int(lp.species[0].Args["Np"]) for lp in self.loops if lp.species)
