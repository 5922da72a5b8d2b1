"""Reverse-mode gradients of a PIC run: the adjoint of ``PIC_loop.step()``.

The reference has no differentiation.  Here a scalar loss of the final
fields -- by default the mean of the on-axis longitudinal field squared,
Ex_m0[1, ix]^2 (x is the propagation axis in these arrays: this is the
plasma wake), over the last ``loss_window`` lambda0 of the window -- is
differentiated with respect to the laser's amplitude a0, waist R and focal
position x_foc, and to the knot values of the longitudinal density profile,
through every step of a moving-window run (injection included).

How.  Each operation of the step (chimeraCL/pic_loop.py:57-142) is linear
in the fields or differentiable in the particles, and has a hand-written
transpose in the library:

* particles: push_xyz (``ccl_push_x_adjoint``), the current and charge
  deposits as gathers of the node adjoints (``ccl_deposit_adjoint``), the
  gather + Boris push reversed with its field adjoints scattered onto the
  nodes (``ccl_gather_push_adjoint``), align as a scatter
  (``ccl_align_adjoint``), the density profile (``ccl_dens_profile_adjoint``);
* fields: the Fourier-Bessel transforms by the same FFT kernels with the
  conjugate phase and the Hankel GEMMs with transposed matrices (for the
  forward FFT F and the backward B = F^H / N: F^T = N B, B^T = F / N), the
  edge damping (self-adjoint: its half transforms transpose into each
  other), the PSATD update (``ccl_psatd_adjoint``), the combine steps of the
  gradient and the curl (``ccl_grad_combine_adjoint``,
  ``ccl_rot_combine_adjoint`` + transposed derivative GEMMs), deposit
  post-processing and ghost rows.

The forward is run once, keeping a checkpoint every ``every`` steps
(``checkpoint.save_checkpoint``).  The reverse sweep restores each
checkpoint in turn, recomputes its steps eagerly while recording what the
transposes read (each step's particles, both cell sorts, the gathered E and
B, the window's injections), and walks those steps backwards.  Injected
coordinates are held fixed (the injector places each slab from the previous
one's last particles, a discontinuous rule); weights carry the density
profile's gradient.  The laser enters through the initial spectral E_z and
G_z of mode 0: their adjoints are contracted on the host, in float64, with
the derivatives of the pulse set-up (``laser.add_gausian_pulse``: Gaussian
envelope, forward transform, analytic focusing).

``PICLoss`` wraps it as a ``torch.autograd.Function``."""
import copy

import numpy as np
import torch

from ._lib import PP, call, ints, longs, stream
from .checkpoint import restore_checkpoint, save_checkpoint
from .methods.generic_methods_cu import LazyScalar
from .methods.solver_methods_cu import psatd_split_coefficients
from .pic_loop import capture_guard

VEC = ("x", "y", "z")


class _Rec:
    """What the reverse sweep reads of one forward step."""


class _Patch:
    """Instance-method wrappers for the duration of a with-block."""

    def __init__(self):
        self.saved = []

    def wrap(self, obj, name, fn):
        self.saved.append((obj, name, obj.__dict__.get(name)))
        setattr(obj, name, fn)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        for obj, name, old in reversed(self.saved):
            if old is None:
                delattr(obj, name)
            else:
                setattr(obj, name, old)


class PICAdjoint:
    """Gradients of a loss of the final fields of ``loop`` (one solver, one
    moving window, mobile species and immobile ones injected from a source
    species) with respect to the laser and the density profile knots.

    ``laser_in``: the dict ``add_gausian_pulse`` was given; ``profile``: the
    density profile dict (coord 'x', points, values) the run used for the
    prefilled domain ``prefill`` and the injections, or None."""

    def __init__(self, loop, laser_in, profile=None, prefill=None, every=10, graphs=True):
        if len(loop.solvers) != 1:
            raise ValueError("the adjoint handles one solver")
        self.loop = loop
        self.S = loop.solvers[0]
        self.laser_in = dict(laser_in)
        if float(self.laser_in.get("astig", 0.0) or 0.0):
            raise ValueError("the adjoint does not cover the astigmatic laser term")
        self.profile = profile
        self.prefill = dict(prefill) if prefill is not None else None
        self.every = int(every)
        # graphs: the recomputation through the loop's CUDA graphs and the
        # reverse step as one graph per epoch (else all eager)
        self.graphs = bool(graphs)
        # profile_phases: time restore / recompute / reverse (synchronising)
        self.profile_phases = False
        self.timing = {}
        self.checkpoints = {}
        # per window-shift step of the forward: each species' in-window count
        # after the shift's align (the recomputation's align takes it from
        # here instead of waiting for the device; checked after the sweep)
        self._shift_counts = {}
        self._count_checks = []
        self.nsteps = 0
        comm = self.S.comm
        self.dt_ccl = comm.ccl
        self.real, self.cplx, self.dev = comm.real, comm.cplx, comm.device
        A = self.S.Args
        self.M, self.Nx, self.Nr = A["M"], A["Nx"], A["Nr"]
        self._prepared = False

    # ------------------------------------------------------------------
    # forward
    def run(self, nsteps):
        """Step the run nsteps times, keeping a checkpoint every `every`."""
        loop = self.loop
        self.it0 = loop.it
        # keep the particle pieces' graphs of every window position of the
        # run: the reverse sweep's recomputation replays them all (each
        # holds its position's particle arrays)
        shifts = [fr.Args["Steps"] for fr in loop.frames]
        epochs = int(nsteps) // max(1, int(min(shifts))) + 2 if shifts else 1
        loop.graph_cache_size = max(loop.graph_cache_size, epochs)
        for _ in range(int(nsteps)):
            if (loop.it - self.it0) % self.every == 0:
                self.checkpoints[loop.it] = save_checkpoint(loop)
            it, shift = loop.it, loop._frame_due()
            loop.step()
            if shift:  # the align left Np = the in-window count (a host int)
                self._shift_counts[it] = {id(p): dict.__getitem__(p.Args, "Np")
                                          for p in loop.species}
        self.nsteps = loop.it - self.it0
        # the final state the loss reads (the reverse sweep leaves the run at
        # its start; gradients() may be called more than once)
        A = self.S.Args
        self._final = {"it": loop.it, "xgrid": np.array(A["Xgrid"], dtype=np.float64),
                       "xmax": float(A["Xmax"]),
                       "ex_row": self.S.DataDev["Ex_m0"][1].to(torch.float64).clone()}
        return loop.it

    @staticmethod
    def _clock():
        import time
        torch.cuda.synchronize()
        return time.perf_counter()

    def _final_state(self):
        """What the loss reads: recorded at the end of run(), else the
        loop's current state."""
        F = getattr(self, "_final", None)
        if F is not None:
            return F
        A = self.S.Args
        return {"it": self.loop.it, "xgrid": np.array(A["Xgrid"], dtype=np.float64),
                "xmax": float(A["Xmax"]),
                "ex_row": self.S.DataDev["Ex_m0"][1].to(torch.float64)}

    def loss_window(self, width):
        """Columns of the last `width` of the window (at the end of run())."""
        F = self._final_state()
        return np.nonzero(F["xgrid"] >= F["xmax"] - width)[0]

    def wake_loss(self, width=20.0):
        """mean(Ex_m0[1, ix]^2) over the last `width` of the window at the end
        of run() (float64)."""
        sel = self._upload(self.loss_window(width), np.int64)
        row = self._final_state()["ex_row"][sel]
        return (row * row).mean()

    # ------------------------------------------------------------------
    # set-up of the transposes
    def _prepare(self):
        if self._prepared:
            return
        S, A, D = self.S, self.S.Args, self.S.DataDev
        M = self.M
        # the transposed matrices and the real coefficient arrays the reverse
        # step reads, held here: a checkpoint restore rebinds the solver's
        # arrays to fresh copies, and a captured reverse step must keep
        # reading the ones it was captured with (names starting with "_" are
        # working arrays that checkpoints leave alone)
        self._const = {k: S._real_dev(k) for k in ["kx", "dV_inv", "DampProfile"] + [
            "%s_m%d" % (n, m) for n in ("SmoothingFilter", "Poiss") for m in range(M + 1)]}
        for m in range(M + 1):
            for name in ("DHT_m", "DHT_inv_m", "dDHT_plus_m", "dDHT_minus_m"):
                key = name + str(m)
                D["_adjT_" + key] = D[key].t().contiguous()
            coef = psatd_split_coefficients(A["w_m" + str(m)], A["dt"])
            D["_adj_psatd_m%d" % m] = torch.as_tensor(np.ascontiguousarray(coef),
                                                      device=self.dev).to(self.real)
        shp = (self.Nr - 1, self.Nx)
        self._spec = lambda: torch.zeros(shp, dtype=self.cplx, device=self.dev)
        self._realsp = lambda m: torch.zeros((self.Nr, self.Nx),
                                             dtype=self.real if m == 0 else self.cplx,
                                             device=self.dev)
        self._work = lambda m: torch.zeros(shp, dtype=self.real if m == 0 else self.cplx,
                                           device=self.dev)
        # the reverse step's buffers, allocated once (per grid)
        n3, spec = 3 * (M + 1), self._spec
        W = self.ws = {}
        W["lEB"] = [self._realsp(m) for m in range(M + 1) for _ in range(6)]
        W["lB"] = [spec() for _ in range(n3)]
        W["lJ"] = [spec() for _ in range(n3)]
        W["ldN_alt"] = [spec() for _ in range(n3)]
        W["lrho"] = [spec() for _ in range(M + 1)]
        W["Pm"] = [spec() if (m > 0 or M > 0) else None for m in range(M + 1)]
        W["Pp"] = [spec() if m < M else None for m in range(M + 1)]
        W["Rm"] = [spec() if t is not None else None for t in W["Pm"]]
        W["Rp"] = [spec() if t is not None else None for t in W["Pp"]]
        W["Qm"] = [spec() if (m > 0 or M > 0) else None for m in range(M + 1) for _ in VEC]
        W["Qp"] = [spec() if m < M else None for m in range(M + 1) for _ in VEC]
        W["Sm"] = [spec() if t is not None else None for t in W["Qm"]]
        W["Sp"] = [spec() if t is not None else None for t in W["Qp"]]
        W["lrho_rs"] = [self._realsp(m) for m in range(M + 1)]
        W["lJ_rs"] = [self._realsp(m) for m in range(M + 1) for _ in VEC]
        W["bwork"] = [self._work(m) for m in range(M + 1) for _ in range(6)]
        W["eout"] = [spec() for _ in range(n3)]
        W["fwork"] = {m: [self._work(m) for _ in range(4)] for m in range(M + 1)}
        W["damp_rs"] = {m: self._realsp(m) for m in range(M + 1)}
        # zeroed before every reverse step: the scattered E, B adjoints and
        # row 0 of the transposed forward transforms' outputs
        zs = [(t, t.numel(), int(t.is_complex())) for t in W["lEB"]]
        zs += [(t[0], t.shape[1], int(t.is_complex())) for t in W["lrho_rs"] + W["lJ_rs"]]
        W["zero"] = zs
        self._phases = {}
        self._prepared = True

    def _phase(self, xmin, sign):
        """exp(sign i kx xmin), kept per origin (the window moves every few
        steps: a few origins per run)."""
        key = (float(xmin), sign)
        buf = self._phases.get(key) if hasattr(self, "_phases") else None
        if buf is None:
            buf = torch.empty(self.Nx, dtype=self.cplx, device=self.dev)
            call("ccl_phase", self.dt_ccl, self.Nx, buf.data_ptr(),
                 self.S.DataDev["kx"].data_ptr(), float(xmin), sign, stream())
            if hasattr(self, "_phases"):
                self._phases[key] = buf
        return buf

    def _zero_ws(self):
        from ._lib import longs as _longs
        z = self.ws["zero"]
        for k in range(0, len(z), 32):
            part = z[k:k + 32]
            call("ccl_set_batch", self.dt_ccl, len(part), ints([c for _, _, c in part]),
                 _longs([n for _, n, _ in part]), PP([t for t, _, _ in part]), 0.0, 0.0,
                 stream())

    def _gemm(self, names, X, Y, cplx_flags, alpha, beta=0.0):
        """Y_i = beta Y_i + alpha A_i^T-named X_i over whole (Nr-1, Nx) fields
        (complex fields as 2 Nx real columns), one batched launch per call;
        entries must not share an output."""
        S = self.S
        nx = self.Nx
        groups = {}
        for n, x, y, c in zip(names, X, Y, cplx_flags):
            groups.setdefault(c, []).append((n, x, y))
        for c, ent in groups.items():
            ncol = 2 * nx if c else nx
            for k in range(0, len(ent), 32):
                part = ent[k:k + 32]
                S._gemm([e[0] for e in part], [e[1] for e in part], [ncol] * len(part),
                         [e[2] for e in part], [ncol] * len(part), [ncol] * len(part),
                         cplx=bool(c), alpha=alpha, beta=beta)

    # ------------------------------------------------------------------
    # recording forward steps (the step of PIC_loop._body, eagerly)
    def _species(self):
        mob = [p for p in self.loop.species if "Immobile" not in p.Args]
        imm = [p for p in self.loop.species if "Immobile" in p.Args]
        return mob, imm

    def _sort_rec(self, p):
        D = p.DataDev
        return (D["sort_indx"].clone(), D["cell_offset"].clone(), D["Np_stay_dev"].clone())

    def _copies(self, pairs):
        """dst <- src for (dst, src) tensor pairs, batched (32 per launch)."""
        pairs = [(d, s_) for d, s_ in pairs if s_.numel()]
        for k in range(0, len(pairs), 32):
            part = pairs[k:k + 32]
            call("ccl_copy_batch", len(part), longs([s_.numel() * s_.element_size()
                                                     for _, s_ in part]),
                 PP([d for d, _ in part]), PP([s_ for _, s_ in part]), stream())

    def _snapshot(self, tensors):
        """Fresh copies of `tensors` (one batched launch); one allocation per
        group of equal shape and dtype (the recording runs on the host's
        clock: an allocation per tensor cost more than the copies)."""
        groups = {}
        for i, t in enumerate(tensors):
            groups.setdefault((t.dtype, tuple(t.shape)), []).append(i)
        out = [None] * len(tensors)
        for (dt, shape), idx in groups.items():
            if len(idx) == 1:
                out[idx[0]] = torch.empty(shape, dtype=dt, device=self.dev)
            else:
                block = torch.empty((len(idx),) + shape, dtype=dt, device=self.dev)
                for i, v in zip(idx, block.unbind(0)):
                    out[i] = v
        self._copies(list(zip(out, tensors)))
        return out

    def _record_step(self, imm_sorts):
        """Step the loop once, recording what the reverse step reads: the
        mobile species' positions, momenta and g_inv at the step's start
        (after the window shift), the positions and cell sort at its end
        (the charge deposit's and the gather's), the gathered E, B (the
        real-space fields at the step's end, ghost rows included), the
        weights, and at a window shift the injection (_frame_recorded).  A
        step without a window shift runs as the loop's own CUDA-graph
        replays."""
        loop, S = self.loop, self.S
        mob, imm = self._species()
        rec = _Rec()
        rec.it = loop.it
        rec.frame = None
        frame = loop._frame_due()
        if frame:
            rec.frame = self._frame_recorded()
            imm_sorts.clear()
        A = S.Args
        rec.xmin = float(A["Xmin"])
        pre_keys = ("x", "y", "z", "px", "py", "pz", "g_inv")
        pre = self._snapshot([p.DataDev[k] for p in mob for k in pre_keys])
        rec.mob = []
        for i, p in enumerate(mob):
            d = dict(zip(pre_keys, pre[7 * i:7 * i + 7]))
            d["w"], d["Np"] = p.DataDev["w"], int(p.Args["Np"])
            rec.mob.append(d)
        rec.imm = [{"x": p.DataDev["x"], "y": p.DataDev["y"], "z": p.DataDev["z"],
                    "w": p.DataDev["w"], "Np": int(p.Args["Np"])} for p in imm]
        if frame and self.graphs:
            # as the loop's own shift step: particle pieces eager, the field
            # solve replayed (phase factors moved first)
            for sol in loop.solvers:
                sol._phase(0)
                sol._phase(1)
            loop._eager_pieces()
            loop._eager_left = 0  # the next steps replay (their graphs are cached)
            loop.it += 1
        elif frame or not self.graphs:
            loop._step_part(graph_mode=False)
            loop.it += 1
        else:
            loop.step()
        D = S.DataDev
        eb = [D[f + c + "_m" + str(m)] for m in range(self.M + 1) for f in ("E", "B")
              for c in VEC]
        post = []
        for p in mob:
            Dp = p.DataDev
            post += [Dp["x"], Dp["y"], Dp["z"], Dp["sort_indx"], Dp["cell_offset"],
                     Dp["Np_stay_dev"]]
        for i, p in enumerate(imm):
            if i not in imm_sorts:
                imm_sorts[i] = tuple(self._snapshot([p.DataDev["sort_indx"],
                                                      p.DataDev["cell_offset"],
                                                      p.DataDev["Np_stay_dev"]]))
        snap = self._snapshot(post + eb)
        rec.X2, rec.sort2 = [], []
        for i in range(len(mob)):
            x, y, z, si, co, ns = snap[6 * i:6 * i + 6]
            rec.X2.append({"x": x, "y": y, "z": z})
            rec.sort2.append((si, co, ns))
        rec.EB = snap[6 * len(mob):]
        rec.imm_sort = [imm_sorts[i] for i in range(len(imm))]
        return rec

    def _frame_recorded(self):
        """The window shift + injection of PIC_loop._frame_part, recording
        each species' injected slab, counts and align permutation."""
        loop = self.loop
        fr = {}

        def rec_of(p):
            return fr.setdefault(id(p), {})

        with _Patch() as pt:
            for p in loop.species:
                def mnd(parts_in, density_profiles=None, _p=p, _f=type(p).make_new_domain):
                    _f(_p, parts_in, density_profiles)
                    r = rec_of(_p)
                    r["dom"] = dict(parts_in)
                    r["profiles"] = density_profiles
                    r["x_new"] = _p.DataDev["x_new"].clone()
                    r["w_new"] = _p.DataDev["w_new"].clone()

                def anp(source=None, _p=p, _f=type(p).add_new_particles):
                    r = rec_of(_p)
                    r["np_old"] = int(_p.Args["Np"])
                    r["source"] = id(source) if source is not None else id(_p)
                    _f(_p, source)

                def rec_align(_p):
                    r = rec_of(_p)
                    r["np_pre"] = int(_p.Args["Np"])
                    known = self._shift_counts.get(loop.it, {}).get(id(_p))
                    lazy = dict.__getitem__(_p.Args, "Np_stay")
                    if isinstance(known, int) and isinstance(lazy, LazyScalar):
                        # the forward's count for this shift: no wait here
                        # (the recomputation is the forward's arithmetic;
                        # gradients() compares the two after the sweep)
                        self._count_checks.append((lazy, known))
                        dict.__setitem__(_p.Args, "Np_stay", known)
                    ns = int(_p.Args["Np_stay"])
                    r["np_stay"] = ns
                    r["sort_indx"] = _p.DataDev["sort_indx"][:ns].clone()

                def alg(_p=p, _f=type(p).align_parts):
                    rec_align(_p)
                    _f(_p)

                def alb(_p=p, _f=getattr(type(p), "align_begin", None)):
                    # (the window shift aligns in two halves; the record is
                    # the same, taken before the permutation)
                    rec_align(_p)
                    _f(_p)
                pt.wrap(p, "make_new_domain", mnd)
                pt.wrap(p, "add_new_particles", anp)
                pt.wrap(p, "align_parts", alg)
                if hasattr(type(p), "align_begin"):
                    pt.wrap(p, "align_begin", alb)
            loop._frame_part()
        return fr

    # ------------------------------------------------------------------
    # the reverse sweep
    def gradients(self, width=20.0, grad_output=1.0):
        """dL/d(a0, R, x_foc) and dL/d(profile values) of L = wake_loss(width)
        (times grad_output), after run()."""
        if not self.checkpoints:
            raise RuntimeError("run() first")
        self._prepare()
        loop, S = self.loop, self.S
        D, A, M = S.DataDev, S.Args, self.M
        final_it = self._final_state()["it"]
        # the loss seed on the final real-space Ex_m0
        sel = self._upload(self.loss_window(width), np.int64)
        seed = torch.zeros(self.Nx, dtype=torch.float64, device=self.dev)
        seed[sel] = 2.0 * self._final_state()["ex_row"][sel] / len(sel) * float(grad_output)
        self._seed = seed.to(self.real)
        self._seed_buf = torch.zeros(self.Nx, dtype=self.real, device=self.dev)
        # adjoint state: spectral E, G, the carried dN1, particles
        self.lE = [self._spec() for _ in range(3 * (M + 1))]
        self.lG = [self._spec() for _ in range(3 * (M + 1))]
        self.ldN = [self._spec() for _ in range(3 * (M + 1))]
        self._graph = None  # (key, CUDA graph) of the current epoch's reverse step
        self._cur = None
        self._warm = False
        mob, imm = self._species()
        self.lmob = [self._particle_adj(int(p.Args["Np"]), True) for p in mob]
        self.limm = [self._particle_adj(int(p.Args["Np"]), False) for p in imm]
        nprof = 0 if self.profile is None else len(self.profile["values"])
        self.lknots = torch.zeros(max(nprof, 1), dtype=torch.float64, device=self.dev)
        starts = sorted(self.checkpoints, reverse=True)
        tm = self.timing = {"restore": 0.0, "recompute": 0.0, "reverse": 0.0}
        clock = self._clock if self.profile_phases else (lambda: 0.0)
        for s in starts:
            e = min(s + self.every, self.it0 + self.nsteps)
            t0 = clock()
            restore_checkpoint(loop, self.checkpoints[s])
            t1 = clock()
            imm_sorts = {}
            recs = [self._record_step(imm_sorts) for _ in range(s, e)]
            t2 = clock()
            for n in range(e - 1, s - 1, -1):
                self._reverse_step(recs[n - s], final=(n == final_it - 1))
                recs[n - s] = None
            del recs
            t3 = clock()
            tm["restore"] += t1 - t0
            tm["recompute"] += t2 - t1
            tm["reverse"] += t3 - t2
        self._graph = None
        self._cur = None
        checks, self._count_checks = self._count_checks, []
        for lazy, known in checks:
            if lazy.resolve() != known:
                raise RuntimeError("adjoint: a recomputed window shift kept %d particles where "
                                   "the forward kept %d" % (lazy.resolve(), known))
        # t = 0: the prefilled particles' weights, the laser
        restore_checkpoint(loop, self.checkpoints[self.it0])
        if self.profile is not None and self.prefill is not None:
            src = mob[0]
            x, w = src.DataDev["x"], src.DataDev["w"]
            lw = self.lmob[0]["w"]
            for r in self.limm:
                lw = lw + r["w"]
            self._knots(self.prefill, x, w, lw)
        g_laser = self._laser_gradient()
        return g_laser, (self.lknots[:nprof].cpu().numpy() if nprof else np.zeros(0))

    def _particle_adj(self, n, mobile):
        z = lambda: torch.zeros(n, dtype=self.real, device=self.dev)
        if not mobile:
            return {"w": z()}
        return {k: z() for k in ("x", "y", "z", "px", "py", "pz", "g_inv", "w")}

    def _gp(self, xmin):
        A = self.S.Args
        return (self.Nx, float(xmin), float(A["dx_inv"]), self.Nr, float(A["Rmin"]),
                float(A["dr_inv"]))

    def _reverse_step(self, rec, final):
        """One step backwards: the step's records copied into the epoch's
        fixed input buffers, then the transposes -- as one CUDA-graph replay
        (captured on the epoch's first step; an epoch is the run between two
        window shifts: particle counts, the grid origin and the particle
        adjoint arrays fixed), eagerly on the very first step (it builds the
        library's lazily created tables and the transposed matrices' split
        forms) -- then, at a window shift, the injection's transpose."""
        mob, imm = self._species()
        key = (tuple(r["Np"] for r in rec.mob), tuple(r["Np"] for r in rec.imm), rec.xmin,
               tuple(id(L["x"]) for L in self.lmob), tuple(id(L["w"]) for L in self.limm))
        if self._cur is None or self._cur["key"] != key:
            self._cur = self._epoch_buffers(rec, key)
            self._graph = None
        cur = self._cur
        # per-step inputs
        pairs = []
        for i, r in enumerate(rec.mob):
            c = cur["mob"][i]
            pairs += [(c[k], r[k]) for k in ("x", "y", "z", "px", "py", "pz", "g_inv", "w")]
            pairs += [(c["x2"], rec.X2[i]["x"]), (c["y2"], rec.X2[i]["y"]),
                      (c["z2"], rec.X2[i]["z"])]
            pairs += list(zip(c["sort2"], rec.sort2[i]))
        pairs += list(zip(cur["EB"], rec.EB))
        for i, r in enumerate(rec.imm):  # the ions change only between segments
            c = cur["imm"][i]
            src = [r["x"], r["y"], r["z"], r["w"]] + list(rec.imm_sort[i])
            if c["src"] != tuple(t.data_ptr() for t in src):
                pairs += list(zip([c["x"], c["y"], c["z"], c["w"]] + list(c["sort"]), src))
                c["src"] = tuple(t.data_ptr() for t in src)
        self._copies(pairs)
        if final:
            self._seed_buf.copy_(self._seed)
        if self._graph is not None:
            self._graph.replay()
        elif not self._warm or not self.graphs:
            self._reverse_body(cur)
            self._warm = True
        else:
            self._phase(cur["xmin"], 1)
            self._phase(cur["xmin"], -1)
            g = torch.cuda.CUDAGraph()
            if getattr(self, "_cap_stream", None) is None:
                self._cap_stream = torch.cuda.Stream()
            now = torch.cuda.current_stream()
            self._cap_stream.wait_stream(now)
            with torch.cuda.stream(self._cap_stream), capture_guard():
                g.capture_begin()
                try:
                    self._reverse_body(cur)
                finally:
                    g.capture_end()
            now.wait_stream(self._cap_stream)
            g.replay()
            self._graph = g
        if final:
            self._seed_buf.zero_()
        if rec.frame is not None:
            self._frame_adj(rec.frame)

    def _epoch_buffers(self, rec, key):
        """Fixed inputs of the reverse step for one epoch (see _reverse_step)
        and the first half push's positions and cell sort."""
        from ._lib import sort_workspace_bytes
        A = self.S.Args
        C = (A["Nx"] - 1) * (A["Nr"] - 1)
        cur = {"key": key, "xmin": rec.xmin, "mob": [], "imm": []}
        for r, X2, s2 in zip(rec.mob, rec.X2, rec.sort2):
            c = {k: torch.empty_like(r[k]) for k in ("x", "y", "z", "px", "py", "pz", "g_inv",
                                                     "w")}
            c.update({k + "2": torch.empty_like(X2[k]) for k in VEC})
            c.update({k + "1": torch.empty_like(X2[k]) for k in VEC})
            c["sort2"] = [torch.empty_like(t) for t in s2]
            n = r["Np"]
            ws_b = sort_workspace_bytes(n, C)
            i32 = lambda k: torch.empty(max(k, 1), dtype=torch.int32, device=self.dev)[:k]
            c["sort1"] = (i32(n), i32(C + 1), i32(C + 2), i32(n), i32(1))
            c["sort_ws"] = (torch.empty(ws_b, dtype=torch.uint8, device=self.dev), ws_b)
            cur["mob"].append(c)
        cur["EB"] = [torch.empty_like(t) for t in rec.EB]
        for r, srt in zip(rec.imm, rec.imm_sort):
            c = {k: torch.empty_like(r[k]) for k in ("x", "y", "z", "w")}
            c["sort"] = [torch.empty_like(t) for t in srt]
            c["src"] = None
            cur["imm"].append(c)
        cur["ldN0"] = [self._spec() for _ in range(3 * (self.M + 1))]
        return cur

    def _reverse_body(self, cur):
        """The transposes of one step, on the epoch's fixed buffers (no host
        reads, no allocation once the caches are warm: capturable)."""
        S, D, M = self.S, self.S.DataDev, self.M
        W = self.ws
        mob, imm = self._species()
        dtc = self.dt_ccl
        nrows, nx = self.Nr - 1, self.Nx
        gp = self._gp(cur["xmin"])
        ppos = self._phase(cur["xmin"], 1)   # exp(+i kx Xmin)
        pneg = self._phase(cur["xmin"], -1)  # exp(-i kx Xmin)
        self._zero_ws()
        # 0. the first half push's positions and their cell sort
        for i, p in enumerate(mob):
            c = cur["mob"][i]
            self._copies([(c["x1"], c["x"]), (c["y1"], c["y"]), (c["z1"], c["z"])])
            call("ccl_push_x", dtc, c["x"].numel(), c["x1"].data_ptr(), c["y1"].data_ptr(),
                 c["z1"].data_ptr(), c["px"].data_ptr(), c["py"].data_ptr(),
                 c["pz"].data_ptr(), c["g_inv"].data_ptr(), float(p.Args["dt_2"]), stream())
            keys, cnt, off, si, ns = c["sort1"]
            ws, ws_b = c["sort_ws"]
            call("ccl_index_sort", dtc, c["x"].numel(), c["x1"].data_ptr(), c["y1"].data_ptr(),
                 c["z1"].data_ptr(), *gp, keys.data_ptr(), cnt.data_ptr(), off.data_ptr(),
                 si.data_ptr(), ns.data_ptr(), ws.data_ptr(), ws_b, stream())
        # 1. gather + push (E, B real-space adjoints; particles)
        lEB = W["lEB"]
        lEB[0][1].add_(self._seed_buf)  # the loss seed (zero but on the final step)
        for i, p in enumerate(mob):
            c, L = cur["mob"][i], self.lmob[i]
            si, co, ns = c["sort2"]
            call("ccl_gather_push_adjoint", dtc, M, c["x2"].data_ptr(), c["y2"].data_ptr(),
                 c["z2"].data_ptr(), c["px"].data_ptr(), c["py"].data_ptr(),
                 c["pz"].data_ptr(), si.data_ptr(), co.data_ptr(), ns.data_ptr(),
                 float(p.Args["FactorPush"]), *gp, PP(cur["EB"]), PP(lEB), L["x"].data_ptr(),
                 L["y"].data_ptr(), L["z"].data_ptr(), L["px"].data_ptr(), L["py"].data_ptr(),
                 L["pz"].data_ptr(), L["g_inv"].data_ptr(), stream())
        # 2. ghost rows
        call("ccl_warp_axis_adjoint", dtc, M, 2 * 3, PP(self._field_major(lEB)), nx, stream())
        # 3. backward transforms of E, B: lE += F(DHT_inv^T lE_rs) / N; lB = the same of lB_rs
        self._backward_transform_adj(lEB, pneg)
        # 4. B = rot(G) / w^2
        self._rot_adj(W["lB"])
        # 5. edge damping (self-adjoint)
        self._damp_adj(ppos, pneg)
        # 6. PSATD (the current's smoothing filter applied to lJ in the same pass)
        lJ, ldN0 = W["lJ"], cur["ldN0"]
        for m in range(M + 1):
            sl = slice(3 * m, 3 * m + 3)
            call("ccl_psatd_adjoint", dtc, nrows * nx, D["_adj_psatd_m%d" % m].data_ptr(),
                 self._const["SmoothingFilter_m%d" % m].data_ptr(),
                 PP(self.lE[sl] + self.lG[sl] + lJ[sl] + ldN0[sl] + self.ldN[sl]), stream())
        # 7. gradient of rho (and rho's smoothing filter): lrho = f grad^T ldN;
        #    then the carried dN adjoint becomes ldN0
        lrho = W["lrho"]
        self._grad_adj(self.ldN, lrho, filt=True)
        self._copies(list(zip(self.ldN, ldN0)))
        # 8. forward transforms of rho, J
        lrho_rs, lJ_rs = W["lrho_rs"], W["lJ_rs"]
        ent = [(m, lrho[m], lrho_rs[m]) for m in range(M + 1)]
        ent += [(m, lJ[3 * m + c], lJ_rs[3 * m + c]) for m in range(M + 1) for c in range(3)]
        self._forward_transform_adj(ent, ppos)
        # 9. deposit post-processing
        dv = self._const["dV_inv"].data_ptr()
        call("ccl_deposit_postproc_adjoint", dtc, M, 1, PP(lrho_rs), nx, self.Nr, dv, stream())
        lJ_fm = [lJ_rs[3 * m + c] for c in range(3) for m in range(M + 1)]
        call("ccl_deposit_postproc_adjoint", dtc, M, 3, PP(lJ_fm), nx, self.Nr, dv, stream())
        # 10. charge deposit at X2 (ions: weights only)
        for i, p in enumerate(mob):
            c = cur["mob"][i]
            si, co, _ = c["sort2"]
            X2 = {"x": c["x2"], "y": c["y2"], "z": c["z2"]}
            self._deposit_adj(False, p, si, co, X2, c, c["w"], lrho_rs, gp, self.lmob[i])
        for i, p in enumerate(imm):
            c = cur["imm"][i]
            si, co, _ = c["sort"]
            self._deposit_adj(False, p, si, co, c, None, c["w"], lrho_rs, gp, self.limm[i],
                              positions=False)
        # 11. second half push
        for i, p in enumerate(mob):
            self._push_adj(p, cur["mob"][i], self.lmob[i])
        # 12. current deposit at X1
        for i, p in enumerate(mob):
            c = cur["mob"][i]
            _, _, off, si, _ = c["sort1"]
            X1 = {"x": c["x1"], "y": c["y1"], "z": c["z1"]}
            self._deposit_adj(True, p, si, off, X1, c, c["w"], lJ_rs, gp, self.lmob[i])
        # 13. first half push
        for i, p in enumerate(mob):
            self._push_adj(p, cur["mob"][i], self.lmob[i])

    def _field_major(self, lEB):
        """m-major (6 per mode: Ex..Bz) -> field-major (E x,y,z then B x,y,z,
        each over modes), the layout of the post-processing / ghost-row
        entry points."""
        M = self.M
        return [lEB[6 * m + 3 * f + c] for f in range(2) for c in range(3) for m in range(M + 1)]

    def _deposit_adj(self, vec, p, si, co, X, r, w, lam, gp, L, positions=True):
        dtc, M = self.dt_ccl, self.M
        lamp = PP(lam)
        u = [r["px"].data_ptr(), r["py"].data_ptr(), r["pz"].data_ptr(),
             r["g_inv"].data_ptr()] if vec else [None] * 4
        lu = [L["px"].data_ptr(), L["py"].data_ptr(), L["pz"].data_ptr(),
              L["g_inv"].data_ptr()] if vec else [None] * 4
        lx = [L["x"].data_ptr(), L["y"].data_ptr(), L["z"].data_ptr()] if positions \
            else [None] * 3
        call("ccl_deposit_adjoint", dtc, int(vec), M, si.data_ptr(), co.data_ptr(),
             X["x"].data_ptr(), X["y"].data_ptr(), X["z"].data_ptr(), *u, w.data_ptr(),
             int(p.Args["charge"]), *gp, lamp, *lx, L["w"].data_ptr(), *lu, stream())

    def _push_adj(self, p, r, L):
        call("ccl_push_x_adjoint", self.dt_ccl, r["px"].numel(), r["px"].data_ptr(),
             r["py"].data_ptr(),
             r["pz"].data_ptr(), r["g_inv"].data_ptr(), L["x"].data_ptr(), L["y"].data_ptr(),
             L["z"].data_ptr(), L["px"].data_ptr(), L["py"].data_ptr(), L["pz"].data_ptr(),
             L["g_inv"].data_ptr(), float(p.Args["dt_2"]), stream())

    # -- transforms ------------------------------------------------------
    def _backward_transform_adj(self, lEB, pneg):
        """The backward transforms of E and B transposed: for each component
        and mode, spec (+)= phase- F(DHT_inv_m^T rs[1:]) / Nx -- added to the
        carried E adjoint, written to the B adjoint (one GEMM launch per
        kind, one FFT launch, one add)."""
        W, M = self.ws, self.M
        dtc, nrows, nx = self.dt_ccl, self.Nr - 1, self.Nx
        ent = []  # (m, real-space adjoint, FFT output)
        for m in range(M + 1):
            for f in range(2):
                for c in range(3):
                    out = (W["eout"] if f == 0 else W["lB"])[3 * m + c]
                    ent.append((m, lEB[6 * m + 3 * f + c], out))
        works = W["bwork"]
        self._gemm(["_adjT_DHT_inv_m%d" % m for m, _, _ in ent],
                   [rs.data_ptr() + nx * rs.element_size() for _, rs, _ in ent],
                   [w.data_ptr() for w in works], [m != 0 for m, _, _ in ent],
                   alpha=1.0 / nx)
        for k in range(0, len(ent), 32):
            e, w = ent[k:k + 32], works[k:k + 32]
            b = len(e)
            call("ccl_fft_forward_batch", dtc, b, nrows, nx, PP(w), longs([nx] * b),
                 ints([int(m == 0) for m, _, _ in e]), PP([o for _, _, o in e]),
                 pneg.data_ptr(), PP([None] * b), stream())
        n = len(self.lE)
        call("ccl_add_batch", dtc, n, longs([2 * t.numel() for t in self.lE]), PP(self.lE),
             PP(W["eout"]), stream())

    def _forward_transform_adj(self, ent, ppos):
        """ent: (m, spectral adjoint, real-space adjoint (Nr, Nx)):
        rs[1:] = Nx DHT_m^T B(spec) with B the backward FFT stage (phase+,
        real part for m = 0); rs[0] is left as it is (zeroed per step).  The
        smoothing filter the forward applied is already in the spectral
        adjoints (psatd and gradient transposes)."""
        dtc, nrows, nx = self.dt_ccl, self.Nr - 1, self.Nx
        pool = {m: list(v) for m, v in self.ws["fwork"].items()}
        works = [pool[m].pop() for m, _, _ in ent]  # one buffer of the entry's kind each
        for k in range(0, len(ent), 32):
            e, w = ent[k:k + 32], works[k:k + 32]
            b = len(e)
            call("ccl_fft_backward_batch", dtc, b, nrows, nx, PP([s for _, s, _ in e]), PP(w),
                 longs([nx] * b), ints([int(m == 0) for m, _, _ in e]), ppos.data_ptr(),
                 stream())
        self._gemm(["_adjT_DHT_m%d" % m for m, _, _ in ent], [w.data_ptr() for w in works],
                   [rs.data_ptr() + nx * rs.element_size() for _, _, rs in ent],
                   [m != 0 for m, _, _ in ent], alpha=float(nx))

    def _damp_adj(self, ppos, pneg):
        S, A, D = self.S, self.S.Args, self.S.DataDev
        M = self.M
        nf = 2 * int(S._damp_cells())
        prof = self._const["DampProfile"]
        ent = [(self.lE[3 * m + c], m) for m in range(M + 1) for c in range(3)]
        ent += [(self.lG[3 * m + c], m) for m in range(M + 1) for c in range(3)]
        scratch = self.ws["damp_rs"]
        for k in range(0, len(ent), 32):
            part = ent[k:k + 32]
            call("ccl_damp_batch", self.dt_ccl, len(part), self.Nr - 1, self.Nx,
                 PP([sp for sp, _ in part]), PP([scratch[m] for _, m in part]),
                 ints([int(m == 0) for _, m in part]), ppos.data_ptr(), pneg.data_ptr(),
                 prof.data_ptr(), nf, stream())

    # -- gradient / curl -------------------------------------------------
    def _grad_adj(self, ldN, lrho, filt=False):
        """lrho = grad^T ldN (times the smoothing filter with filt)."""
        S, M, dtc, W = self.S, self.M, self.dt_ccl, self.ws
        nrows, nx = self.Nr - 1, self.Nx
        Pm, Pp = W["Pm"], W["Pp"]
        call("ccl_grad_combine_adjoint", dtc, M, nrows, nx, self._const["kx"].data_ptr(),
             PP(ldN), PP(lrho), PP(Pm), PP(Pp), stream())
        Rm, Rp = self._products_T(Pm, Pp, W["Rm"], W["Rp"])
        fl = PP([self._const["SmoothingFilter_m%d" % m] for m in range(M + 1)]) if filt else None
        call("ccl_modes_adjoint_accumulate", dtc, M, 1, nrows, nx, PP(lrho), PP(Rm), PP(Rp),
             fl, stream())

    def _rot_adj(self, lB):
        S, M, dtc, W = self.S, self.M, self.dt_ccl, self.ws
        nrows, nx = self.Nr - 1, self.Nx
        Qm, Qp = W["Qm"], W["Qp"]
        poiss = [self._const["Poiss_m%d" % m] for m in range(M + 1)]
        call("ccl_rot_combine_adjoint", dtc, M, nrows, nx, self._const["kx"].data_ptr(),
             PP(poiss), PP(lB), PP(self.lG), PP(Qm), PP(Qp), stream())
        Rm, Rp = self._products_T(Qm, Qp, W["Sm"], W["Sp"], ncomp=3)
        call("ccl_modes_adjoint_accumulate", dtc, M, 3, nrows, nx, PP(self.lG), PP(Rm), PP(Rp),
             None, stream())

    def _products_T(self, Pm, Pp, Rm, Rp, ncomp=1):
        """Rm[i] = dDHT_minus_m^T Pm[i], Rp[i] = dDHT_plus_m^T Pp[i] (i =
        ncomp m + c) into the given outputs, one batched GEMM."""
        names, X, Y = [], [], []
        for lst, out, base in ((Pm, Rm, "_adjT_dDHT_minus_m%d"), (Pp, Rp, "_adjT_dDHT_plus_m%d")):
            for i, t in enumerate(lst):
                if t is None:
                    continue
                names.append(base % (i // ncomp))
                X.append(t.data_ptr())
                Y.append(out[i].data_ptr())
        self._gemm(names, X, Y, [True] * len(names), alpha=1.0)
        return Rm, Rp

    # -- window shift + injection ------------------------------------------
    def _frame_adj(self, fr):
        mob, imm = self._species()
        dtc = self.dt_ccl
        src_new = {}
        for p in mob + imm:
            r = fr[id(p)]
            if "x_new" in r:
                src_new[id(p)] = r
        for lst, species in ((self.lmob, mob), (self.limm, imm)):
            for i, p in enumerate(species):
                r = fr[id(p)]
                L = lst[i]
                pre = {k: torch.zeros(r["np_pre"], dtype=self.real, device=self.dev) for k in L}
                keys = list(L)
                call("ccl_align_adjoint", dtc, r["np_stay"], len(keys), PP([L[k] for k in keys]),
                     PP([pre[k] for k in keys]), r["sort_indx"].data_ptr(), stream())
                n0 = r["np_old"]
                lst[i] = {k: v[:n0].clone() for k, v in pre.items()}
                inj = src_new.get(r["source"])
                if inj is not None and self.profile is not None and inj["profiles"]:
                    self._knots(inj["dom"], inj["x_new"], inj["w_new"], pre["w"][n0:].contiguous())

    def _upload(self, a, dtype=np.float64):
        """A host array on the device, through pinned memory: a copy from
        pageable memory would wait for the whole reverse sweep queued so
        far."""
        h = torch.from_numpy(np.ascontiguousarray(a, dtype=dtype))
        if torch.device(self.dev).type != "cuda":
            return h.to(self.dev)
        return h.pin_memory().to(self.dev, non_blocking=True)

    def _knots(self, dom, x, w, lw):
        """Accumulate the profile-knot adjoints of the weights w = w0 f(x) of
        particles placed in the domain `dom` (the knots dens_profile used)."""
        prf = self.profile
        xp = np.array(prf["points"], dtype=np.double)
        fp = np.array(prf["values"], dtype=np.double)
        i0 = int((xp < dom["Xmin"]).sum() - 1)
        i1 = int((xp < dom["Xmax"]).sum() + 1)
        xl, fl = xp[i0:i1], fp[i0:i1]
        dxm1 = 1.0 / (xl[1:] - xl[:-1])
        xl_d, fl_d, dx_d = (self._upload(a) for a in (xl, fl, dxm1))
        out = torch.zeros(len(xl), dtype=torch.float64, device=self.dev)
        call("ccl_dens_profile_adjoint", self.dt_ccl, x.numel(), x.data_ptr(), w.data_ptr(),
             lw.data_ptr(), xl_d.data_ptr(), fl_d.data_ptr(), dx_d.data_ptr(), len(xl),
             out.data_ptr(), stream())
        self.lknots[i0:i0 + len(xl)] += out

    # -- laser -------------------------------------------------------------
    def _laser_gradient(self):
        """dL/d(a0, R, x_foc): the t = 0 adjoints of Ez_fb_m0 and Gz_fb_m0
        contracted (float64, host) with the derivatives of the pulse set-up
        of laser.add_gausian_pulse."""
        S, A = self.S, self.S.Args
        L = self.laser_in
        k0 = 2 * np.pi * L["k0"]
        a0, Lx, R, x0, x_foc = L["a0"], L["Lx"], L["R"], L["x0"], L["x_foc"]
        X = x0 - x_foc
        Xg, Rg = A["Xgrid"], A["Rgrid"]
        kx, w = A["kx"][None, :], A["w_m0"]
        r1 = Rg[1:, None]
        ez = (a0 * np.sin(k0 * (Xg[None, :] - x0))
              * np.exp(-(Xg[None, :] - x0) ** 2 / Lx ** 2 - r1 ** 2 / R ** 2)
              * (abs(r1) < 3.5 * R) * (abs(Xg[None, :] - x0) < 3.5 * Lx))
        phs = np.exp(-1j * A["kx"] * float(A["Xmin"]))[None, :]
        dht = S.DataDev["DHT_m0"].to(torch.float64).cpu().numpy()

        def fb(f):  # forward transform of a mode-0 real field, rows 1..
            return np.fft.fft(dht.dot(f), axis=1) * phs

        def focus(EE):
            DT = -1.0j * w * np.sign(kx + (kx == 0))
            GG0 = DT * EE
            e = np.exp(1.0j * kx * X)
            cw, sw = np.cos(w * X), np.sin(w * X)
            E1 = e * (cw * EE + sw / w * GG0)
            G1 = e * (-w * sw * EE + cw * GG0)
            dE = 1.0j * kx * E1 + e * (-w * sw * EE + cw * GG0)
            dG = 1.0j * kx * G1 + e * (-w * w * cw * EE - w * sw * GG0)
            return E1, G1, dE, dG

        EE = fb(ez)
        lE = self.lE[2].cpu().numpy().astype(np.complex128)   # Ez, m = 0
        lG = self.lG[2].cpu().numpy().astype(np.complex128)   # Gz, m = 0

        def contract(dE, dG):
            return float(np.real(np.conj(lE) * dE).sum() + np.real(np.conj(lG) * dG).sum())

        _, _, dEX, dGX = focus(EE)
        E_a, G_a, _, _ = focus(EE / a0)
        E_R, G_R, _, _ = focus(fb(ez * 2 * r1 ** 2 / R ** 3))
        return np.array([contract(E_a, G_a), contract(E_R, G_R), -contract(dEX, dGX)])


# ----------------------------------------------------------------------
class PICLoss(torch.autograd.Function):
    """loss = PICLoss.apply(params, knots, problem): params = (a0, R, x_foc)
    and knots = the density profile's values (float64 tensors), `problem` a
    dict describing the run (see ``build_problem_run``).  The forward runs
    the simulation with a checkpoint every problem['every'] steps and
    returns the wake loss; backward runs the adjoint sweep."""

    @staticmethod
    def forward(ctx, params, knots, problem):
        run = build_problem_run(problem, params.detach().cpu().numpy(),
                                knots.detach().cpu().numpy())
        adj = run["adjoint"]
        adj.run(problem["nsteps"])
        loss = adj.wake_loss(problem.get("loss_width", 20.0))
        ctx.adj = adj
        ctx.width = problem.get("loss_width", 20.0)
        ctx.shapes = (params.shape, knots.shape, params.dtype, params.device)
        return loss.detach().cpu()

    @staticmethod
    def backward(ctx, grad):
        g_laser, g_knots = ctx.adj.gradients(ctx.width, float(grad))
        shp_p, shp_k, dt, dev = ctx.shapes
        gp = torch.as_tensor(g_laser, dtype=dt, device=dev).reshape(shp_p)
        gk = torch.as_tensor(g_knots, dtype=dt, device=dev).reshape(shp_k)
        ctx.adj = None
        return gp, gk, None


def build_problem_run(problem, params, knots):
    """Set the run of `problem` up through the public API with laser
    parameters params = (a0, R, x_foc) and density knot values `knots`:
    problem = {grid_in, eons_in, frame_in, laser_in (k0, x0, Lx), prefill,
    knot_points, precision, seed, nsteps, every[, loss_width]}."""
    from . import Communicator
    from .frame import Frame
    from .laser import add_gausian_pulse
    from .particles import Particles
    from .pic_loop import PIC_loop
    from .solver import Solver

    a0, R, x_foc = (float(v) for v in params)
    laser = dict(problem["laser_in"], a0=a0, R=R, x_foc=x_foc)
    profile = {"coord": "x", "points": list(map(float, problem["knot_points"])),
               "values": list(map(float, knots))}
    comm = Communicator(precision=problem.get("precision", "mixed"), seed=problem["seed"],
                        device=problem.get("device", 0))
    solver = Solver(copy.deepcopy(problem["grid_in"]), comm)
    add_gausian_pulse(solver, dict(laser))
    e_in = copy.deepcopy(problem["eons_in"])
    e_in.update(dx=solver.Args["dx"], dr=solver.Args["dr"], dt=solver.Args["dt"])
    i_in = copy.deepcopy(e_in)
    i_in["charge"] = 1
    i_in["Immobile"] = True
    eons = Particles(e_in, comm, seed=problem["seed"])
    ions = Particles(i_in, comm, seed=problem["seed"] + 1)
    ions.Args["InjectorSource"] = eons
    eons.make_new_domain(dict(problem["prefill"]), density_profiles=[profile])
    eons.add_new_particles()
    ions.add_new_particles(source=eons)
    eons.free_added()
    f_in = dict(problem["frame_in"], dt=solver.Args["dt"], DensityProfiles=[profile])
    loop = PIC_loop([solver], [eons, ions], [Frame(f_in)], graphs=problem.get("graphs", True))
    adj = PICAdjoint(loop, laser, profile=profile, prefill=problem["prefill"],
                     every=problem.get("every", 10), graphs=problem.get("adjoint_graphs", True))
    return {"solver": solver, "eons": eons, "ions": ions, "loop": loop, "adjoint": adj}


def differentiable_problem(seed=0, nsteps=100, precision="mixed", Nx=1024, Nr=128, nknots=32,
                           every=10):
    """The differentiable run: the 512 x 64 LPA run's window (z in [-40, 0],
    r in [0, 20] lambda0) on Nx x Nr = 1024 x 128, m = 0, 1, 2x2x4
    macro-electrons per cell, immobile ions, laser a0 = 2, w0 = 6, tau = 5
    (field FWHM) centred and focused at z = -10, moving window with injection
    every 20 steps, absorbing edges of min(50, Nx/8) cells, nsteps steps
    with a checkpoint every `every`; the
    density n_e = 1e-3 n_c times a piecewise-linear profile through `nknots`
    knots spanning [-42, 6] lambda0 (past both ends of every slab the run
    injects) with values drawn uniformly in [0.5, 2] from `seed`.  Returns
    (problem, params0 = (a0, R, x_foc), knots0)."""
    rng = np.random.default_rng(seed)
    knots = rng.uniform(0.5, 2.0, nknots)
    points = np.linspace(-42.0, 6.0, nknots)
    tau = 5.0
    problem = dict(
        grid_in=dict(Xmin=-40.0, Xmax=0.0, Nx=Nx, Rmin=0.0, Rmax=20.0, Nr=Nr, M=1,
                     DampCells=min(50, Nx // 8)),
        eons_in=dict(Nppc=(2, 2, 4), dens=1e-3, charge=-1),
        frame_in=dict(Velocity=1.0, Steps=20),
        laser_in=dict(k0=1.0, x0=-10.0, Lx=tau / (2 * np.sqrt(np.log(2)))),
        prefill=dict(Xmin=-40.0, Xmax=0.0, Rmin=0.0, Rmax=20.0),
        knot_points=points, precision=precision, seed=seed, nsteps=nsteps, every=every,
        loss_width=20.0)
    return problem, np.array([2.0, 6.0, -10.0]), knots
