"""Particle methods (the CUDA counterpart of
chimeraCL/methods/particles_methods_cl.py): coordinate push, cell sort,
align, plasma/beam injection."""
import numpy as np
import torch

from .._lib import CCL_F64, PP, call, sort_workspace_bytes, stream
from .generic_methods_cu import GenericMethodsCU, LazyScalar


def injector_last_columns(Xg, npx):
    """x of the particle columns of an injected slab's last two cells, last
    column first, in the injector's double arithmetic (particles_generic.cl:
    62-74, x = xmin + ((0.5 + ixx) * (1/npx)) * Lx): the values whose FP32
    rounding the slab stores there.  The last cell can fall outside the
    window and be dropped, hence two."""
    Nx_loc = len(Xg)
    return [float(Xg[ix] + (0.5 + ixx) * (1.0 / npx) * (Xg[ix + 1] - Xg[ix]))
            for ix in (Nx_loc - 2, Nx_loc - 3) if ix >= 0
            for ixx in range(npx - 1, -1, -1)]


class ParticleMethodsCU(GenericMethodsCU):
    def init_particle_methods(self):
        self.init_generic_methods()
        # Host generator of the injector's random draws (the reference uses a
        # device Threefry stream, particles_methods_cl.py:22): PCG64, seeded,
        # so that runs are reproducible and comparable draw for draw.
        seed = getattr(self, "_seed", None)
        if seed is None:
            seed = self.comm.seed
        self._rng = np.random.Generator(np.random.PCG64(seed))

    def _comps(self):
        if "Immobile" in self.Args:
            comps = ["x", "y", "z", "w"]
        else:
            comps = ["x", "y", "z", "px", "py", "pz", "w", "g_inv"]
        if self.comm.compensated:
            # immobile species too: their charge must sit where the mobile
            # species' charge sits (ions are injected on the electrons)
            comps += ["x_lo", "y_lo", "z_lo"]
        return comps

    def _new_low_parts(self, Np):
        """Zero low parts of the coordinates of Np new particles (filled in
        by the injector where its positions are not FP32 values)."""
        if "x_lo" in self._comps():
            for arg in ("x_lo", "y_lo", "z_lo"):
                self.DataDev[arg + "_new"] = torch.zeros(Np, dtype=self.comm.real,
                                                         device=self.comm.device)

    def add_new_particles(self, source=None):
        """particles_methods_cl.py:40-64"""
        src = self.DataDev if source is None else source.DataDev
        for arg in self._comps():
            self.DataDev[arg] = torch.cat([self.DataDev[arg], src[arg + "_new"]])
        self.reset_num_parts()
        self.flag_sorted = False

    def make_new_domain(self, parts_in, density_profiles=None):
        """particles_methods_cl.py:66-147"""
        A, D = self.Args, self.DataDev
        xmin, xmax, rmin, rmax = (parts_in[k] for k in ("Xmin", "Xmax", "Rmin", "Rmax"))
        Nx_loc = int(np.ceil((xmax - xmin) / A["dx"]) + 1)
        Nr_loc = int(np.round((rmax - rmin) / A["dr"]) + 1)
        Xg = xmin + A["dx"] * np.arange(Nx_loc)
        Rg = rmin + A["dr"] * np.arange(Nr_loc)
        A["right_lim"] = Xg[-1]
        # candidates for the next right limit of FP32 coordinates
        A["_inj_last_x"] = injector_last_columns(Xg, int(A["Nppc"][0]))
        ncells = (Nx_loc - 1) * (Nr_loc - 1)
        Np = int(ncells * np.prod(A["Nppc"]))
        real = self.comm.real
        for arg in ("x", "y", "z", "w"):
            D[arg + "_new"] = torch.empty(Np, dtype=real, device=self.comm.device)
        self._new_low_parts(Np)
        theta = self.dev_arr(shape=ncells, dtype=np.double)
        self._fill_arr_rand(theta, xmin=0, xmax=2 * np.pi)
        Xg_d, Rg_d = self.dev_arr(val=Xg), self.dev_arr(val=Rg)
        npx, npr, npth = (int(v) for v in A["Nppc"])
        if "x_lo_new" in D:
            # compensated FP32 coordinates: the positions in double (the FP64
            # injector's values), split into FP32 value + FP32 residual
            f64 = [torch.empty(Np, dtype=torch.float64, device=self.comm.device)
                   for _ in range(4)]
            call("ccl_fill_grid", CCL_F64, ncells, *[t.data_ptr() for t in f64],
                 theta.data_ptr(), Xg_d.data_ptr(), Rg_d.data_ptr(), Nx_loc, npx, npr, npth,
                 stream())
            for arg, t in zip(("x", "y", "z"), f64):
                D[arg + "_new"].copy_(t)
                D[arg + "_lo_new"].copy_(t - D[arg + "_new"].to(torch.float64))
            D["w_new"].copy_(f64[3])
        else:
            call("ccl_fill_grid", self._dt, ncells, D["x_new"].data_ptr(),
                 D["y_new"].data_ptr(), D["z_new"].data_ptr(), D["w_new"].data_ptr(),
                 theta.data_ptr(), Xg_d.data_ptr(), Rg_d.data_ptr(), Nx_loc, npx, npr, npth,
                 stream())
        D["w_new"] *= A["w0"]
        if density_profiles is not None:
            for prf in density_profiles:
                if prf["coord"] != "x":
                    print("Only longitudinal profiling is implemented")
                    continue
                self.dens_profile(prf["points"], prf["values"], parts_in["Xmin"],
                                  parts_in["Xmax"], coord=prf["coord"] + "_new", weight="w_new")
        if "Immobile" not in A:
            for arg in ("px", "py", "pz"):
                if "d" + arg not in parts_in and arg + "_c" not in parts_in:
                    D[arg + "_new"] = torch.zeros(Np, dtype=real, device=self.comm.device)
                    parts_in[arg + "_c"] = 0
                    parts_in["d" + arg] = 0
                else:
                    D[arg + "_new"] = torch.empty(Np, dtype=real, device=self.comm.device)
                    parts_in.setdefault(arg + "_c", 0)
                    if "d" + arg in parts_in:
                        self._fill_arr_randn(D[arg + "_new"], mu=parts_in[arg + "_c"],
                                             sigma=parts_in["d" + arg])
                    else:
                        parts_in["d" + arg] = 0
                        D[arg + "_new"].fill_(parts_in[arg + "_c"])
            mom = sum(parts_in[k] ** 2 for k in ("px_c", "py_c", "pz_c", "dpx", "dpy", "dpz"))
            D["g_inv_new"] = torch.ones(Np, dtype=real, device=self.comm.device)
            if mom != 0:
                call("ccl_gamma_inv", self._dt, Np, D["px_new"].data_ptr(),
                     D["py_new"].data_ptr(), D["pz_new"].data_ptr(), D["g_inv_new"].data_ptr(),
                     stream())

    def make_new_beam(self, parts_in):
        """particles_methods_cl.py:149-177 (normal draws in the order
        x, y, z, px, py, pz)."""
        D, Np = self.DataDev, int(parts_in["Np"])
        real = self.comm.real
        for arg in ("x", "y", "z", "px", "py", "pz", "w"):
            D[arg + "_new"] = torch.empty(Np, dtype=real, device=self.comm.device)
        self._new_low_parts(Np)
        for arg in ("x", "y", "z"):
            v = self._fill_arr_randn(D[arg + "_new"], mu=parts_in[arg + "_c"],
                                     sigma=parts_in["L" + arg])
            if arg + "_lo_new" in D:  # the draws' FP32 rounding residual
                self._upload(D[arg + "_lo_new"], v - v.astype(np.float32).astype(np.float64))
        for arg in ("px", "py", "pz"):
            parts_in.setdefault(arg + "_c", 0)
            parts_in.setdefault("d" + arg, 0)
            self._fill_arr_randn(D[arg + "_new"], mu=parts_in[arg + "_c"], sigma=parts_in["d" + arg])
        D["w_new"].fill_(parts_in["FullCharge"] / parts_in["Np"])
        D["g_inv_new"] = torch.empty(Np, dtype=real, device=self.comm.device)
        call("ccl_gamma_inv", self._dt, Np, D["px_new"].data_ptr(), D["py_new"].data_ptr(),
             D["pz_new"].data_ptr(), D["g_inv_new"].data_ptr(), stream())

    def dens_profile(self, x_prf, f_prf, xmin, xmax, coord="x", weight="w"):
        """particles_methods_cl.py:179-204"""
        x_prf = np.array(x_prf, dtype=np.double)
        f_prf = np.array(f_prf, dtype=np.double)
        i0 = (x_prf < xmin).sum() - 1
        i1 = (x_prf < xmax).sum() + 1
        x_loc = x_prf[i0:i1]
        f_loc = f_prf[i0:i1]
        if x_loc.size < 2:
            raise ValueError("dens_profile: the profile knots must bracket the domain "
                             f"[{xmin}, {xmax}]")
        dxm1 = 1.0 / (x_loc[1:] - x_loc[:-1])
        xl, fl, dl = self.dev_arr(val=x_loc), self.dev_arr(val=f_loc), self.dev_arr(val=dxm1)
        D = self.DataDev
        call("ccl_dens_profile", self._dt, D[coord].numel(), D[coord].data_ptr(),
             D[weight].data_ptr(), xl.data_ptr(), fl.data_ptr(), dl.data_ptr(), x_loc.size,
             stream())

    def push_coords(self, mode="half", sort_grid=None):
        """particles_methods_cl.py:206-223.  With ``sort_grid`` the push
        also forms the cell keys and counts of the sort on that grid from the
        coordinates it has just computed (one kernel); the next
        ``index_sort`` on the same grid then only completes the sort."""
        self._keys_for = None
        if self.Args["Np"] == 0 or "Immobile" in self.Args:
            return
        D = self.DataDev
        dt = self.Args["dt_2"] if mode == "half" else self.Args["dt"]
        lo = [D[k].data_ptr() for k in ("x_lo", "y_lo", "z_lo")] if "x_lo" in D else None
        if sort_grid is not None:
            bufs, G = self._sort_buffers(sort_grid), sort_grid.Args
            call("ccl_push_x_keys", self._dt, self.Args["Np"], D["x"].data_ptr(),
                 D["y"].data_ptr(), D["z"].data_ptr(), *(lo or [None] * 3),
                 *[D[k].data_ptr() for k in ("px", "py", "pz", "g_inv")], float(dt),
                 G["Nx"], float(G["Xmin"]), float(G["dx_inv"]), G["Nr"], float(G["Rmin"]),
                 float(G["dr_inv"]), D["indx_in_cell"].data_ptr(),
                 D["sum_in_cell"].data_ptr(), bufs[5].data_ptr(), bufs[6], stream())
            self._keys_for = self._sort_token(sort_grid)
        elif lo is not None:
            call("ccl_push_x_compensated", self._dt, self.Args["Np"],
                 *[D[k].data_ptr() for k in ("x", "y", "z")], *lo,
                 *[D[k].data_ptr() for k in ("px", "py", "pz", "g_inv")], float(dt), stream())
        else:
            call("ccl_push_x", self._dt, self.Args["Np"], D["x"].data_ptr(), D["y"].data_ptr(),
                 D["z"].data_ptr(), D["px"].data_ptr(), D["py"].data_ptr(), D["pz"].data_ptr(),
                 D["g_inv"].data_ptr(), float(dt), stream())
        self.flag_sorted = False

    def _sort_token(self, grid):
        """What the keys depend on besides the coordinates: the particle
        arrays, their count and the grid."""
        G, D = grid.Args, self.DataDev
        return (self.Args["Np"], D["x"].data_ptr(), G["Nx"], G["Nr"], float(G["Xmin"]),
                float(G["dx_inv"]), float(G["Rmin"]), float(G["dr_inv"]))

    def _sort_buffers(self, grid):
        """The sort's outputs and workspace; they persist while Np and the
        grid are unchanged, so a step between window shifts allocates nothing
        (and can be graph-captured)."""
        Np = self.Args["Np"]
        C = grid.Args["Nxm1Nrm1"]
        dev, D = self.comm.device, self.DataDev
        key = (Np, C)
        bufs = getattr(self, "_sort_bufs", None)
        if bufs is None or bufs[0] != key:
            i32 = torch.int32
            ws_bytes = sort_workspace_bytes(Np, C)
            bufs = (key, torch.empty(max(Np, 1), dtype=i32, device=dev)[:Np],
                    torch.empty(C + 1, dtype=i32, device=dev),
                    torch.empty(C + 2, dtype=i32, device=dev),
                    torch.empty(max(Np, 1), dtype=i32, device=dev)[:Np],
                    torch.empty(ws_bytes, dtype=torch.uint8, device=dev), ws_bytes)
            self._sort_bufs = bufs
        _, D["indx_in_cell"], D["sum_in_cell"], D["cell_offset"], D["sort_indx"] = bufs[:5]
        return bufs

    def index_sort(self, grid):
        """particles_methods_cl.py:225-261: keys, counts, exclusive prefix
        (cell_offset), stable sort -- one C-ABI call, or the completion of
        the sort whose keys the coordinate push formed.  Np_stay stays on
        the device (read lazily through Args)."""
        bufs = self._sort_buffers(grid)
        D, G, Np = self.DataDev, grid.Args, self.Args["Np"]
        ws, ws_bytes = bufs[5], bufs[6]
        if getattr(self, "_keys_for", None) == self._sort_token(grid):
            call("ccl_index_sort_keyed", Np, G["Nx"], G["Nr"], D["indx_in_cell"].data_ptr(),
                 D["sum_in_cell"].data_ptr(), D["cell_offset"].data_ptr(),
                 D["sort_indx"].data_ptr(), D["Np_stay_dev"].data_ptr(), ws.data_ptr(),
                 ws_bytes, stream())
        else:
            call("ccl_index_sort", self._dt, Np, D["x"].data_ptr(), D["y"].data_ptr(),
                 D["z"].data_ptr(), G["Nx"], float(G["Xmin"]), float(G["dx_inv"]), G["Nr"],
                 float(G["Rmin"]), float(G["dr_inv"]), D["indx_in_cell"].data_ptr(),
                 D["sum_in_cell"].data_ptr(), D["cell_offset"].data_ptr(),
                 D["sort_indx"].data_ptr(), D["Np_stay_dev"].data_ptr(), ws.data_ptr(),
                 ws_bytes, stream())
        self._keys_for = None
        dict.__setitem__(self.Args, "Np_stay", LazyScalar(D["Np_stay_dev"], self.comm))

    def align_and_damp(self, comps_align):
        """particles_methods_cl.py:263-286, in two halves (align_queue,
        align_finish): every particle is permuted into cell order -- the
        out-of-window ones last, as the sort leaves them -- before the
        in-window count is read, so the copies are queued while the host
        still runs ahead of the device; after the read the arrays only become
        views of their first Np_stay entries."""
        self.align_finish(self.align_queue(comps_align))

    def align_queue(self, comps_align):
        D = self.DataDev
        Np = self.Args["Np"]
        if Np == 0:
            return comps_align, None, None
        src = [D[c] for c in comps_align]
        # one allocation for all the components (they share one dtype)
        dtypes = {t.dtype for t in src}
        if len(dtypes) == 1:
            block = torch.empty(len(src) * Np, dtype=dtypes.pop(), device=self.comm.device)
            dst = list(block.view(len(src), Np).unbind(0))
        else:
            dst = [torch.empty(Np, dtype=t.dtype, device=self.comm.device) for t in src]
        call("ccl_align", self._dt, Np, len(src), PP(src), PP(dst), D["sort_indx"].data_ptr(),
             stream())
        order = torch.empty(Np, dtype=torch.int32, device=self.comm.device)
        call("ccl_iota_u32", order.data_ptr(), Np, stream())
        return comps_align, dst, order

    def align_finish(self, state):
        comps_align, dst, order = state
        D = self.DataDev
        ns = self.Args["Np_stay"]
        if ns == 0 or dst is None:
            for comp in comps_align + ["sort_indx"]:
                D[comp] = D[comp][:0].clone()
            self.reset_num_parts()
            return
        for c, t in zip(comps_align, dst):
            D[c] = t[:ns]
        D["sort_indx"] = order[:ns]
        self.reset_num_parts()

    def reset_num_parts(self, Np=None):
        """particles_methods_cl.py:288-293"""
        if Np is None:
            Np = self.DataDev["x"].numel()
        self.DataDev["Np"].fill_(Np)
        self.DataDev["Np_stay_dev"].fill_(Np)
        self.Args["Np"] = Np
        self.Args["Np_stay"] = Np

    def _fill_arr_randn(self, arr, mu=0, sigma=1):
        v = mu + sigma * self._rng.standard_normal(arr.numel())
        self._upload(arr, v)
        return v

    def _fill_arr_rand(self, arr, xmin=0, xmax=1):
        v = xmin + (xmax - xmin) * self._rng.random(arr.numel())
        self._upload(arr, v)

    def _upload(self, arr, v):
        """Host draws -> device, through pinned memory and without waiting
        for the device (the pinned block is held until the copy is done)."""
        h = torch.from_numpy(v).to(arr.dtype).pin_memory()
        self.comm.h2d_bytes += h.numel() * h.element_size()
        arr.copy_(h, non_blocking=True)

    def _cumsum(self, arr_in, allocator=None, output_dtype=np.uint32):
        """[0, cumsum(arr_in)...] (particles_methods_cl.py:303-311)."""
        out = torch.zeros(arr_in.numel() + 1, dtype=torch.int64, device=arr_in.device)
        out[1:] = torch.cumsum(arr_in.to(torch.int64), 0)
        return out.to(torch.int32 if np.dtype(output_dtype) == np.uint32 else torch.int64)

    def free_mp(self):
        """Memory pools are torch's caching allocator: nothing to release."""

    def free_added(self):
        for arg in self._comps():
            self.DataDev.pop(arg + "_new", None)
