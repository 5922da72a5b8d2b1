"""The particle-in-cell loop (the reference's chimeraCL/pic_loop.py).

``PIC_loop.step()`` runs the reference's sequence (pic_loop.py:57-142):
frame shift + injection every ``Steps``; half push + sort; current deposit;
half push + sort; charge deposit; forward transforms of rho, J with the
smoothing filter; dN0 <- dN1; spectral grad rho -> dN1; PSATD push; edge
damping; B from G; backward transforms of E, B; gather + Boris push.

With ``timit=True`` each phase is timed on the device with CUDA events under
the reference's twelve phase names (device time, no host synchronisation
inside the step; ``Timer`` is filled when read through ``timings()``).

With ``graphs=True`` the step runs as three CUDA graphs replayed in order:
the particle work before the field solve (pushes, sorts, deposits), the
field solve (transforms, gradient, PSATD push, damping, B, backward
transforms) and the gather + push.  Each is captured on first use and
replayed while a signature of what its launches depend on is unchanged:
device buffers, particle counts and the grid origin for the particle
pieces; the solver's buffers alone for the field piece.  A window shift
(host-driven injection, new particle counts and origin) therefore runs the
particle pieces eagerly for a few steps and then captures them again --
the field solve, ~65 of the step's library calls, is replayed through the
shift (its phase factors are refreshed in place first)."""
import collections
import contextlib
import gc

import numpy as np
import torch

# captures kept per piece (the signatures of the last few window positions)
GRAPH_CACHE = 4

loop_steps = ["frame", "push-x", "sort", "depose", "transform", "smooth", "data_copy",
              "grad", "push-eb", "damp-eb", "restore_B", "gather + push-p"]


@contextlib.contextmanager
def capture_guard():
    """Around a CUDA graph capture: no cyclic garbage collection inside it.
    A collection there could free an unreachable graph of an earlier run,
    and freeing a graph (its memory pool) is not allowed while a capture is
    open -- the capture would be invalidated."""
    was = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if was:
            gc.enable()


def timer_plot(Timer):
    import matplotlib.pyplot as plt
    fig, ax = plt.subplots(figsize=(16, 5))
    keys = list(Timer.keys())
    ind = np.arange(1, len(keys) + 1)
    plt.bar(ind, [Timer[k] for k in keys])
    ax.set_xticks(ind)
    ax.set_xticklabels(keys)
    return fig


class PIC_loop:
    def __init__(self, solvers=(), species=(), frames=(), diags=(), timit=False,
                 fuse_smooth=True, graphs=False):
        self.solvers = list(solvers)
        self.mainsolver = self.solvers[0]
        self.species = list(species)
        self.frames = list(frames)
        self.diags = list(diags)
        self.timit = timit
        # fuse_smooth: apply the smoothing filter inside the forward FFT of
        # rho and J (same arithmetic as fields_smooth after the transform)
        self.fuse_smooth = fuse_smooth
        self.it = 0
        self.Timer = {k: 0.0 for k in loop_steps}
        self._events = []
        self.graphs = graphs
        # piece name -> [graph, signature, library kernels in it] (the one in
        # use), and per piece the last graph_cache_size captures by
        # signature: a run restored to an earlier step (a recompute from a
        # checkpoint) finds the graphs of that stretch of the window again
        self._graphs = {}
        self._graph_cache = {}
        self.graph_cache_size = GRAPH_CACHE
        # steps after a window shift that still launch the particle pieces
        # eagerly before they are captured again (see step())
        self.eager_after_shift = 2
        self._eager_left = 0
        self.graph_replays = 0  # steps served by graph replays
        self.graph_captures = 0  # pieces captured
        self._cap_stream = None
        # library kernels captured / replayed in total (a replay runs the
        # captured kernels without launching them again)
        self.graph_kernels_captured = 0
        self.graph_kernels_replayed = 0

    def timer_start(self):
        if self.timit:
            self._t0 = torch.cuda.Event(enable_timing=True)
            self._t0.record()

    def timer_record(self, name):
        if self.timit:
            e = torch.cuda.Event(enable_timing=True)
            e.record()
            self._events.append((name, self._t0, e))

    def timings(self):
        """Accumulated device time per phase in seconds."""
        if self._events:
            torch.cuda.synchronize()
            for name, a, b in self._events:
                self.Timer[name] += a.elapsed_time(b) * 1e-3
            self._events = []
        return self.Timer

    def _frame_due(self):
        return any(np.mod(self.it, fr.Args["Steps"]) == 0 for fr in self.frames)

    def _signature(self, piece):
        """What a piece's launches depend on: the identity of every device
        buffer (DataDev entries are rebound, never resized in place), the
        particle counts and the grid origin (the field piece: the solvers'
        buffers alone).  Returns (key, refs): comparing keys is a tuple of
        ints; the graph keeps refs, so that no id is reused while it lives."""
        objs = list(self.solvers) + ([] if piece == "f" else list(self.species))
        # (phs_shft names whichever phase buffer was used last)
        refs = tuple(v for obj in objs for k, v in obj.DataDev.items() if k != "phs_shft")
        key = [tuple(map(id, refs))]
        if piece != "f":
            key += [obj.Args.get("Np", None) if hasattr(obj.Args, "get") else None
                    for obj in objs]
            key += [float(sol.Args["Xmin"]) for sol in self.solvers]
        return tuple(key), refs

    def _piece_fn(self, piece):
        return {"pa": self._particles_before, "f": self._fields,
                "pb": self._particles_after}[piece]

    def step(self):
        for diag in self.diags:
            diag.make_record(self.it)
        use_graph = self.graphs and not self.timit and not self.diags and self.it > 0
        if not use_graph:
            self._graphs = {}
            self._graph_cache = {}
            self._eager_left = 0
            self._body(graph_mode=False)
        elif self._frame_due():
            # a window shift: host-driven injection, new particle counts and
            # origin.  The host had to wait for the device (the in-window
            # counts), so it is no longer ahead: the particle pieces run
            # eagerly on this step and the next eager_after_shift ones --
            # each eager step puts the host further ahead, the device being
            # slower than the launches -- and are captured again after that,
            # when the capture's host time overlaps the device's queue.  The
            # field solve replays throughout (its phase factors moved first)
            self._frame_part()
            for sol in self.solvers:
                sol._phase(0)
                sol._phase(1)
            self._eager_left = self.eager_after_shift
            self._eager_pieces()
            if self._eager_left == 0:
                full = self._signature("pa")
                for piece in ("pa", "pb"):
                    if not self._from_cache(piece, full):
                        self._capture(piece)
        elif self._eager_left > 0:
            self._eager_left -= 1
            self._eager_pieces()
        else:
            full = self._signature("pa")  # the same for both particle pieces
            for piece in ("pa", "f", "pb"):
                self._run_piece(piece, full if piece != "f" else None)
            self.graph_replays += 1
        self.it += 1
        return self.it

    def _eager_pieces(self):
        """One graph-mode step with the particle pieces launched eagerly."""
        self._particles_before(graph_mode=True)
        self._run_piece("f")
        self._particles_after(graph_mode=True)
        self.graph_replays += 1

    def _run_piece(self, piece, sig=None):
        g = self._graphs.get(piece)
        sig = sig or self._signature(piece)
        if g is None or sig[0] != g[1][0]:
            if not self._from_cache(piece, sig):
                self._capture(piece)
            g = self._graphs[piece]
        g[0].replay()
        self.graph_kernels_replayed += g[2]

    def _from_cache(self, piece, sig):
        """Make a cached capture of `piece` with this signature the one in
        use; False when there is none."""
        cache = self._graph_cache.get(piece)
        g = cache.get(sig[0]) if cache else None
        if g is None:
            return False
        cache.move_to_end(sig[0])
        self._graphs[piece] = g
        return True

    def _capture(self, piece):
        """Capture one piece of the step into a CUDA graph, on a persistent
        side stream with the graph's own memory pool; unlike
        torch.cuda.graph() this neither synchronises the device nor empties
        the allocator's cache."""
        from . import _lib
        self._graphs.pop(piece, None)
        if piece == "f":
            # phase factors for the current origin, outside the graph: a
            # captured recomputation would replay the capture's origin
            for sol in self.solvers:
                sol._phase(0)
                sol._phase(1)
        n0 = _lib.launch_count()
        g = torch.cuda.CUDAGraph()
        if self._cap_stream is None:
            self._cap_stream = torch.cuda.Stream()
        cur = torch.cuda.current_stream()
        self._cap_stream.wait_stream(cur)
        with torch.cuda.stream(self._cap_stream), capture_guard():
            g.capture_begin()
            try:
                self._piece_fn(piece)(graph_mode=True)
            finally:
                g.capture_end()
        cur.wait_stream(self._cap_stream)
        nk = _lib.launch_count() - n0
        entry = self._graphs[piece] = [g, self._signature(piece), nk]
        cache = self._graph_cache.setdefault(piece, collections.OrderedDict())
        cache[entry[1][0]] = entry
        while len(cache) > self.graph_cache_size:
            cache.popitem(last=False)
        self.graph_captures += 1
        self.graph_kernels_captured += nk

    def _body(self, graph_mode):
        self._frame_part()
        self._step_part(graph_mode)

    def _frame_part(self):
        self.timer_start()
        for frame in self.frames:
            if np.mod(self.it, frame.Args["Steps"]) == 0:
                frame.shift_grids(grids=self.solvers)
                frame.inject_plasma(species=self.species, grid=self.mainsolver)
        self.timer_record("frame")

    def _step_part(self, graph_mode):
        self._particles_before(graph_mode)
        self._fields(graph_mode)
        self._particles_after(graph_mode)

    def _particles_before(self, graph_mode):
        """Half push + sort, current deposit, half push + sort, charge
        deposit (pic_loop.py:73-98).  Each push also forms the sort's cell
        keys from the coordinates it computes (one kernel, no re-read)."""
        for parts in self.species:
            self.timer_start()
            parts.push_coords(mode="half", sort_grid=self.mainsolver)
            self.timer_record("push-x")
            self.timer_start()
            parts.sort_parts(grid=self.mainsolver)
            self.timer_record("sort")

        self.timer_start()
        for solver in self.solvers:
            # rho is cleared here with J (one launch); the charge deposit
            # below then adds onto it
            solver.depose_currents(species=self.species, also_zero=("rho",))
        self.timer_record("depose")

        for parts in self.species:
            self.timer_start()
            parts.push_coords(mode="half", sort_grid=self.mainsolver)
            self.timer_record("push-x")
            self.timer_start()
            parts.sort_parts(grid=self.mainsolver)
            self.timer_record("sort")

        for solver in self.solvers:
            self.timer_start()
            solver.depose_charge(species=self.species, zero=False)
            self.timer_record("depose")

    def _fields(self, graph_mode):
        """Forward transforms with smoothing, dN0 <- dN1, gradient, PSATD
        push, damping, B, backward transforms (pic_loop.py:100-135): reads
        and writes the solver's buffers only."""
        for solver in self.solvers:
            self.timer_start()
            M = solver.Args["M"]
            if self.fuse_smooth:
                filt = [solver._real_dev("SmoothingFilter_m" + str(m)) for m in range(M + 1)]
                solver.fb_transform(scals=["rho"], vects=["J"], dir=0, filt=filt)
                self.timer_record("transform")
            else:
                solver.fb_transform(scals=["rho"], vects=["J"], dir=0)
                self.timer_record("transform")
                self.timer_start()
                solver.fields_smooth(flds=["rho", "Jx", "Jy", "Jz"])
                self.timer_record("smooth")

            # dN0 <- dN1 (pic_loop.py:106-111).  Eagerly the buffers are
            # exchanged (field_grad overwrites dN1 entirely); a captured graph
            # would freeze one exchange, so graph mode copies as the
            # reference does.
            self.timer_start()
            D = solver.DataDev
            for m in range(M + 1):
                for c in solver.Args["vec_comps"]:
                    s = c + "_fb_m" + str(m)
                    if graph_mode:
                        D["dN0" + s].copy_(D["dN1" + s])
                    else:
                        D["dN0" + s], D["dN1" + s] = D["dN1" + s], D["dN0" + s]
            self.timer_record("data_copy")

            self.timer_start()
            solver.field_grad("rho", "dN1")
            self.timer_record("grad")
            self.timer_start()
            solver.push_fields()
            self.timer_record("push-eb")
            self.timer_start()
            solver.damp_fields()
            self.timer_record("damp-eb")
            self.timer_start()
            solver.restore_B_fb()
            self.timer_record("restore_B")
            self.timer_start()
            solver.fb_transform(vects=["E", "B"], dir=1)
            self.timer_record("transform")

    def _particles_after(self, graph_mode):
        """Ghost rows of E, B, gather + Boris push (pic_loop.py:137-142)."""
        for solver in self.solvers:
            self.timer_start()
            solver.gather_and_push(species=self.species)
            self.timer_record("gather + push-p")
        for parts in self.species:
            parts.free_mp()
