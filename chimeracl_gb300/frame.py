"""Moving window (the reference's chimeraCL/frame.py): grid shift and
plasma injection into the uncovered slab."""
import numpy as np
import torch

from .methods.generic_methods_cu import LazyScalar


class TailLimit(LazyScalar):
    """The injector's right limit (frame.py:56-64 of the reference): the
    largest x of the last Nppc+1 particles after the align, plus ddx/2.  The
    tail's few coordinates go to pinned host memory by one asynchronous copy
    when the limit is formed; the arithmetic -- x (+ x_lo) in double, the
    maximum, and for plain FP32 coordinates the snap to the injector's own
    double value of a slab column whose FP32 rounding is that maximum (an
    FP32 right limit would shift every later slab by its rounding) -- runs
    on the host when the next window shift reads it, in the same IEEE
    double operations the device would do.  Forming it costs the shift a
    copy instead of a dozen small device operations, and reading it waits
    for nothing."""

    def __init__(self, x, x_lo, nppc, half_ddx, cand, comm=None):
        tails = [x[-nppc:]] + ([x_lo[-nppc:]] if x_lo is not None else [])
        self._tails = []
        for t in tails:
            h = torch.empty(t.shape, dtype=t.dtype, pin_memory=t.is_cuda)
            h.copy_(t, non_blocking=t.is_cuda)
            self._tails.append(h)
        super().__init__(self._tails[0], comm, float)  # (holds the tail, not the array)
        self._event = None
        if x.is_cuda:
            self._event = torch.cuda.Event()
            self._event.record()
        self._half_ddx = float(half_ddx)
        self._cand = None if cand is None else np.asarray(cand, dtype=np.float64)

    def resolve(self):
        if self.comm is not None:
            self.comm.d2h_bytes += sum(h.numel() * h.element_size() for h in self._tails)
        if self._event is not None:
            self._event.synchronize()
        xs = self._tails[0].numpy()
        xt = xs.astype(np.float64)
        if len(self._tails) > 1:
            xt = xt + self._tails[1].numpy().astype(np.float64)
        x_max = xt.max()
        if self._cand is not None and self._cand.size:
            same = xs.max() == self._cand.astype(np.float32)
            if same.any():
                x_max = self._cand[int(np.argmax(same))]  # the last column wins
        return float(x_max + self._half_ddx)


class Frame:
    def __init__(self, configs_in, comm=None):
        self._process_configs(configs_in)

    def _process_configs(self, configs_in):
        self.Args = configs_in
        self.Args.setdefault("Steps", 1.0)
        self.Args.setdefault("Velocity", 0.0)
        self.Args.setdefault("dt", 1)
        self.Args.setdefault("DensityProfiles", None)

    def shift_grids(self, grids=(), steps=None):
        """Xmin, Xmax, Xgrid += Steps*dt*V on host and device (frame.py:22-30);
        the spectral transforms pick the shift up as the phase exp(i kx Xmin)."""
        if steps is None:
            steps = self.Args["Steps"]
        x_shift = steps * self.Args["dt"] * self.Args["Velocity"]
        for grid in grids:
            for store in (grid.Args, grid.DataDev):
                for arg in ("Xmax", "Xmin", "Xgrid"):
                    store[arg] += x_shift

    def inject_plasma(self, species, grid, steps=None):
        """Fill the slab behind the right edge, then sort, align and find the
        new right limit of each species (frame.py:32-64)."""
        if steps is None:
            steps = self.Args["Steps"]
        x_shift = steps * self.Args["dt"] * self.Args["Velocity"]
        for sp in species:
            if "InjectorSource" in sp.Args:
                # a species injected from a source takes the source's new
                # slab; the reference also generates a slab of its own here
                # and discards it (its draws reach nothing)
                sp.add_new_particles(sp.Args["InjectorSource"])
                continue
            if sp.Args["Np"] == 0:
                sp.Args["right_lim"] = grid.Args["Xmax"] - x_shift
            dom = {"Xmin": sp.Args["right_lim"]}
            dom["Xmax"] = dom["Xmin"] + x_shift
            dom["Rmin"] = grid.Args["Rmin"] * (grid.Args["Rmin"] > 0)
            dom["Rmax"] = grid.Args["Rmax"]
            sp.make_new_domain(dom, density_profiles=self.Args["DensityProfiles"])
            sp.add_new_particles()
        # every species sorted, and its permutation queued, before the first
        # in-window count is read: one wait for the device, and the host work
        # after it is only the arrays' cut to their counts
        for sp in species:
            sp.free_added()
            sp.sort_parts(grid=grid)
        two_halves = all(hasattr(sp, "align_begin") for sp in species)
        for sp in species:
            if two_halves:
                sp.align_begin()
        for sp in species:
            if two_halves:
                sp.align_end()
            else:
                sp.align_parts()
            # right_lim = max x of the last Nppc+1 particles + ddx/2 (with
            # compensated coordinates x is x + x_lo: the next slab is then
            # placed where the FP64 run places it; from a rounded x the whole
            # slab would shift by that rounding), formed on the host from a
            # pinned copy of the tail (TailLimit)
            if sp.Args["Np"] > 0 and "InjectorSource" not in sp.Args:
                nppc = int(np.prod(sp.Args["Nppc"]) + 1)
                x = sp.DataDev["x"]
                x_lo = sp.DataDev.get("x_lo")
                cand = (sp.Args["_inj_last_x"] if x.dtype == torch.float32 and x_lo is None
                        and "_inj_last_x" in sp.Args else None)
                dict.__setitem__(sp.Args, "right_lim",
                                 TailLimit(x, x_lo, nppc, 0.5 * sp.Args["ddx"], cand, sp.comm))
