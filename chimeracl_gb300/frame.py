"""Moving window (the reference's chimeraCL/frame.py): grid shift and
plasma injection into the uncovered slab."""
import numpy as np
import torch

from .methods.generic_methods_cu import LazyScalar


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
        # every species sorted before any is aligned: the first align reads
        # the in-window counts of all of them after one wait for the device
        for sp in species:
            sp.free_added()
            sp.sort_parts(grid=grid)
        for sp in species:
            sp.align_parts()
            # right_lim = max x of the last Nppc+1 particles + ddx/2, formed
            # on the device and copied to pinned host memory at once (the
            # value is the same double sum): neither this step nor the next
            # shift, which reads it, waits for the device.  With
            # compensated coordinates x is x + x_lo: the next slab is then
            # placed where the FP64 run places it (from a rounded x the whole
            # slab would shift by that rounding)
            if sp.Args["Np"] > 0 and "InjectorSource" not in sp.Args:
                nppc = int(np.prod(sp.Args["Nppc"]) + 1)
                x = sp.DataDev["x"]
                x_tail = x[-nppc:].to(torch.float64)
                if "x_lo" in sp.DataDev:
                    x_tail = x_tail + sp.DataDev["x_lo"][-nppc:].to(torch.float64)
                x_max = x_tail.max()
                if x.dtype == torch.float32 and "x_lo" not in sp.DataDev and \
                        "_inj_last_x" in sp.Args:
                    # FP32 coordinates: the last particles are normally the
                    # fresh slab's last columns; where the maximum is one of
                    # those columns' FP32 value, take the double value it
                    # rounds (an FP32 right limit would shift every later
                    # slab by its rounding)
                    # (the candidates travel by one asynchronous pinned copy)
                    cand = torch.tensor(sp.Args["_inj_last_x"], dtype=torch.float64)
                    if x.is_cuda:
                        cand = cand.pin_memory().to(x.device, non_blocking=True)
                    same = x[-nppc:].max() == cand.to(torch.float32)
                    first = torch.argmax(same.to(torch.int32))  # the last column wins
                    x_max = torch.where(same.any(), cand[first], x_max)
                dict.__setitem__(sp.Args, "right_lim",
                                 LazyScalar(x_max + 0.5 * sp.Args["ddx"], sp.comm, float,
                                            prefetch=True))
