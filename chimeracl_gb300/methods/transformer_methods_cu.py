"""Fourier-Bessel transform methods (the CUDA counterpart of
chimeraCL/methods/transformer_methods_cl.py).

A full transform is the batched radial Hankel GEMM (``ccl_dht_gemm``) and the
batched longitudinal FFT (``ccl_fft_forward_rows`` / ``_backward_rows``) with
the moving-window phase, real-part cast and (optionally) the smoothing filter
applied inside the FFT kernel; the half transforms are the FFT kernel alone.
"""
import torch

from .._lib import PP, P, call, ints, longs, stream
from .generic_methods_cu import GenericMethodsCU

MAX_BATCH = 32


class TransformerMethodsCU(GenericMethodsCU):
    def init_transformer_methods(self):
        self.init_generic_methods()
        self._phs_cache = {}
        self._prepare_fft()
        self._prepare_dot()

    # ------------------------------------------------------------------
    def _phase(self, dir):
        """exp(+i kx Xmin) for dir=1, exp(-i kx Xmin) for dir=0
        (get_phase_plus/minus), recomputed only when Xmin moves."""
        x0 = float(self.Args["Xmin"])
        key = (dir, x0)
        t = self._phs_cache.get(dir)
        if t is None or t[0] != x0:
            buf = self.DataDev.get("phs_shft_" + str(dir))
            if buf is None:
                buf = torch.empty(self.Args["Nx"], dtype=self.comm.cplx, device=self.comm.device)
                self.DataDev["phs_shft_" + str(dir)] = buf
            call("ccl_phase", self._dt, self.Args["Nx"], buf.data_ptr(),
                 self.DataDev["kx"].data_ptr(), x0, 1 if dir == 1 else -1, stream())
            self._phs_cache[dir] = (x0, buf)
        self.DataDev["phs_shft"] = self._phs_cache[dir][1]
        del key
        return self._phs_cache[dir][1]

    def _prepare_fft(self):
        """Nothing to plan ahead: FFT plans and twiddle tables are built by
        the library on first use of each length."""

    def _prepare_dot(self):
        """The Hankel GEMM needs no preparation; matrices are uploaded by
        send_args_to_dev."""

    def _bf16x3(self, name):
        """Split, tiled bf16 hi/lo form of a Hankel-type matrix for the
        tensor-core GEMM (built once per matrix)."""
        key = "_bf16x3_" + name
        t = self.DataDev.get(key)
        if t is None:
            import ctypes
            A = self.DataDev[name]
            m, k = A.shape
            nb = ctypes.c_size_t(0)
            call("ccl_dht_bf16x3_prepare_bytes", m, k, ctypes.byref(nb))
            t = torch.empty(nb.value, dtype=torch.uint8, device=self.comm.device)
            call("ccl_dht_bf16x3_prepare", self._ccl_of(A), A.data_ptr(), m, k, t.data_ptr(),
                 nb.value, stream())
            self.DataDev[key] = t
        return t

    def _gemm(self, names, X, ldx, Y, ldy, ncols, cplx=False, alpha=1.0, beta=0.0):
        """Y[i] = beta Y[i] + alpha (A[i] X[i]) for the matrices `names`
        (pointers X, Y as ints), one launch: the BF16x3 tensor-core kernel in
        the mixed form when m, k <= 512 and the rows are 16-byte aligned,
        else the SIMT kernel in the compute precision."""
        a = complex(alpha)
        m, k = self.DataDev[names[0]].shape
        b = len(names)
        if (self.comm.dht_impl == "bf16x3" and k <= 512 and m <= 512
                and all(p % 16 == 0 for p in X) and all(l % 4 == 0 for l in ldx)):
            mats = [self._bf16x3(n) for n in names]
            call("ccl_dht_bf16x3_gemm_batch", b, m, k, ints(ncols), int(cplx), PP(mats), PP(X),
                 longs(ldx), PP(Y), longs(ldy), a.real, a.imag, float(beta), stream())
        else:
            mats = [self._real_dev(n) for n in names]
            call("ccl_dht_gemm_batch", self._dt, b, m, k, ints(ncols), int(cplx), PP(mats), PP(X),
                 longs(ldx), PP(Y), longs(ldy), a.real, a.imag, float(beta), stream())

    def _dht(self, Y, A, X, ldx, ldy, ncols, cplx, alpha=1.0, beta=0.0, xoff=0, yoff=0):
        """Y = beta*Y + alpha*(A X) on one matrix pair; A given by name
        (offsets in elements of the tensors' own dtype)."""
        xp = X.data_ptr() + xoff * X.element_size()
        yp = Y.data_ptr() + yoff * Y.element_size()
        self._gemm([A], [xp], [ldx], [yp], [ldy], [ncols], cplx, alpha, beta)

    def _cdot(self, out, A, X):
        """out = A X for a complex (Nr-1, Nx) field and the matrix named A
        (the reference's _cdot)."""
        nx = X.shape[-1]
        self._dht(out, A, X, 2 * nx, 2 * nx, 2 * nx, True)

    def _ddot(self, out, A, X):
        nx = X.shape[-1]
        self._dht(out, A, X, nx, nx, nx, False)

    # ------------------------------------------------------------------
    def transform_field(self, arg_cmp, dir, mode, filt=None):
        """transformer_methods_cl.py:38-64.  ``filt`` (optional, a list of
        M+1 real filters) multiplies the forward result in the FFT epilogue,
        which is fields_smooth fused into the transform."""
        A = self.Args
        phs = self._phase(dir)
        M, Nx, Nr = A["M"], A["Nx"], A["Nr"]
        nrows = Nr - 1
        for m in range(M + 1):
            s = str(m)
            rs = self.DataDev[arg_cmp + "_m" + s]
            sp = self.DataDev[arg_cmp + "_fb_m" + s]
            if dir == 0:
                f = None if filt is None else filt[m]
                fptr = None if f is None else f.data_ptr()
                if mode == "full":
                    mat = "DHT_m" + s
                    if m == 0:
                        buf = self.DataDev["fld_buff1_d"]
                        self._dht(buf, mat, rs, Nx, Nx, Nx, False, xoff=Nx)
                        call("ccl_fft_forward_rows", self._dt, nrows, Nx, buf.data_ptr(), Nx, 1,
                             sp.data_ptr(), phs.data_ptr(), fptr, stream())
                    else:
                        self._dht(sp, mat, rs, 2 * Nx, 2 * Nx, 2 * Nx, True, xoff=Nx)
                        call("ccl_fft_forward_rows", self._dt, nrows, Nx, sp.data_ptr(), Nx, 0,
                             sp.data_ptr(), phs.data_ptr(), fptr, stream())
                else:
                    call("ccl_fft_forward_rows", self._dt, nrows, Nx, P(rs, Nx), Nx,
                         int(m == 0), sp.data_ptr(), phs.data_ptr(), fptr, stream())
            else:
                if mode == "full":
                    mat = "DHT_inv_m" + s
                    if m == 0:
                        buf = self.DataDev["fld_buff0_d"]
                        call("ccl_fft_backward_rows", self._dt, nrows, Nx, sp.data_ptr(),
                             buf.data_ptr(), Nx, 1, phs.data_ptr(), stream())
                        self._dht(rs, mat, buf, Nx, Nx, Nx, False, yoff=Nx)
                    else:
                        buf = self.DataDev["fld_buff0_c"]
                        call("ccl_fft_backward_rows", self._dt, nrows, Nx, sp.data_ptr(),
                             buf.data_ptr(), Nx, 0, phs.data_ptr(), stream())
                        self._dht(rs, mat, buf, 2 * Nx, 2 * Nx, 2 * Nx, True, yoff=Nx)
                else:
                    call("ccl_fft_backward_rows", self._dt, nrows, Nx, sp.data_ptr(), P(rs, Nx),
                         Nx, int(m == 0), phs.data_ptr(), stream())

    def _work(self, i, cplx):
        """Per-entry work buffer (Nr-1, Nx) of a batched transform."""
        key = ("_wc%d" if cplx else "_wr%d") % i
        buf = self.DataDev.get(key)
        if buf is None:
            shape = (self.Args["Nr"] - 1, self.Args["Nx"])
            buf = torch.empty(shape, dtype=self.comm.cplx if cplx else self.comm.real,
                              device=self.comm.device)
            self.DataDev[key] = buf
        return buf

    def transform_fields(self, names, dir, mode, filt=None):
        """Full or half transforms of several fields at once: every
        (field, mode) pair of a direction shares one Hankel GEMM launch and
        one FFT launch (the same arithmetic as transform_field per pair)."""
        A = self.Args
        M, Nx, Nr = A["M"], A["Nx"], A["Nr"]
        nrows = Nr - 1
        ent = [(n, m) for n in names for m in range(M + 1)]
        for k in range(0, len(ent), MAX_BATCH):
            self._transform_batch(ent[k:k + MAX_BATCH], dir, mode, filt, M, Nx, nrows)

    def _transform_batch(self, ent, dir, mode, filt, M, Nx, nrows):
        D = self.DataDev
        phs = self._phase(dir)
        rs = [D[n + "_m" + str(m)] for n, m in ent]
        sp = [D[n + "_fb_m" + str(m)] for n, m in ent]
        real = [int(m == 0) for _, m in ent]
        ncol = [Nx if m == 0 else 2 * Nx for _, m in ent]
        rows1 = [t.data_ptr() + Nx * t.element_size() for t in rs]  # rows 1..Nr-1
        b = len(ent)
        if dir == 0:
            fl = [None if filt is None else filt[m] for _, m in ent]
            if mode == "full":
                outg = [self._work(i, False) if m == 0 else sp[i] for i, (_, m) in enumerate(ent)]
                self._gemm(["DHT_m" + str(m) for _, m in ent], rows1, ncol,
                           [t.data_ptr() for t in outg], ncol, ncol)
                fin = outg
            else:
                fin = rows1
            call("ccl_fft_forward_batch", self._dt, b, nrows, Nx, PP(fin), longs([Nx] * b),
                 ints(real), PP(sp), phs.data_ptr(), PP(fl), stream())
        else:
            if mode == "full":
                bufs = [self._work(i, m != 0) for i, (_, m) in enumerate(ent)]
                call("ccl_fft_backward_batch", self._dt, b, nrows, Nx, PP(sp), PP(bufs),
                     longs([Nx] * b), ints(real), phs.data_ptr(), stream())
                self._gemm(["DHT_inv_m" + str(m) for _, m in ent],
                           [t.data_ptr() for t in bufs], ncol, rows1, ncol, ncol)
            else:
                call("ccl_fft_backward_batch", self._dt, b, nrows, Nx, PP(sp), PP(rows1),
                     longs([Nx] * b), ints(real), phs.data_ptr(), stream())

    def _transform_forward(self, dht_arg, arg_in, arg_out, phs_shft):
        self.transform_field(arg_in[:-2], 0, "full")

    def _transform_backward(self, dht_arg, arg_in, arg_out, phs_shft):
        self.transform_field(arg_out[:-2], 1, "full")

    def _half_transform_forward(self, dht_arg, arg_in, arg_out, phs_shft):
        self.transform_field(arg_in[:-2], 0, "half")

    def _half_transform_backward(self, dht_arg, arg_in, arg_out, phs_shft):
        self.transform_field(arg_out[:-2], 1, "half")

    # ------------------------------------------------------------------
    def field_poiss_vec(self, fld):
        """B_m *= 1/w^2 (transformer_methods_cl.py:66-71)"""
        for m in range(self.Args["M"] + 1):
            for c in self.Args["vec_comps"]:
                self.mult_elementwise(self._real_dev("Poiss_m" + str(m)),
                                      self.DataDev[fld + c + "_fb_m" + str(m)])

    def field_poiss_scl(self, fld):
        for m in range(self.Args["M"] + 1):
            self.mult_elementwise(self._real_dev("Poiss_m" + str(m)),
                                  self.DataDev[fld + "_fb_m" + str(m)])

    def fields_smooth(self, flds):
        """transformer_methods_cl.py:79-85"""
        for m in range(self.Args["M"] + 1):
            for fld in flds:
                self.mult_elementwise(self._real_dev("SmoothingFilter_m" + str(m)),
                                      self.DataDev[fld + "_fb_m" + str(m)])

    def _get_mm1_vec(self, fld):
        if self.Args["M"] == 0:
            return
        for c in self.Args["vec_comps"]:
            self._get_mm1_one(fld + c, c)

    def _get_mm1_scl(self, fld, comp="x"):
        if self.Args["M"] == 0:
            return
        self._get_mm1_one(fld, comp)

    def _get_mm1_one(self, fld, comp):
        A = self.Args
        call("ccl_get_m1", self._dt, A["Nr"] - 1, A["Nx"],
             self.DataDev["buff_fb_m-1_" + comp].data_ptr(),
             self.DataDev[fld + "_fb_m1"].data_ptr(), stream())

    def _products(self, terms):
        """One batched GEMM launch: out_i = D_i X_i for the (matrix name, X)
        pairs of ``terms`` (None entries skipped); returns the outputs in
        order (None where the term is None)."""
        A = self.Args
        nx = A["Nx"]
        live = [(i, t) for i, t in enumerate(terms) if t is not None]
        outs = [None] * len(terms)
        for k in range(0, len(live), MAX_BATCH):
            part = live[k:k + MAX_BATCH]
            bufs = [self._work(j, True) for j in range(k, k + len(part))]
            self._gemm([t[0] for _, t in part], [t[1].data_ptr() for _, t in part],
                       [2 * nx] * len(part), [b.data_ptr() for b in bufs], [2 * nx] * len(part),
                       [2 * nx] * len(part))
            for (i, _), b in zip(part, bufs):
                outs[i] = b
        return outs

    def field_grad(self, scl_in, vec_out):
        """Spectral gradient (transformer_methods_cl.py:87-133): the
        radial-derivative products of every mode in one batched GEMM, then one
        combine kernel (i kx term, m=-1 mirror, mode coupling)."""
        A, D = self.Args, self.DataDev
        M = A["M"]
        f = [D[scl_in + "_fb_m" + str(m)] for m in range(M + 1)]
        pm = [(("dDHT_minus_m%d" % m), f[m - 1] if m > 0 else f[1])
              if (m > 0 or M > 0) else None for m in range(M + 1)]
        pp = [("dDHT_plus_m%d" % m, f[m + 1]) if m < M else None for m in range(M + 1)]
        prods = self._products(pm + pp)
        out = [D[vec_out + c + "_fb_m" + str(m)] for m in range(M + 1) for c in A["vec_comps"]]
        call("ccl_grad_combine", self._dt, M, A["Nr"] - 1, A["Nx"],
             self._real_dev("kx").data_ptr(), PP(f), PP(prods[:M + 1]), PP(prods[M + 1:]),
             PP(out), stream())

    def field_div(self, vec_in, scl_out):
        """Spectral divergence (transformer_methods_cl.py:135-183)."""
        A, D = self.Args, self.DataDev
        M = A["M"]
        kx = self._real_dev("kx")
        b0, b1 = D["fld_buff0_c"], D["fld_buff1_c"]
        for c in ("y", "z"):
            self._get_mm1_scl(vec_in + c, c)
        for m in range(M + 1):
            s = str(m)
            out = D[scl_out + "_fb_m" + s]
            self.set_to(out, 0.0)
            self.ab_dot_x(1j, kx, D[vec_in + "x_fb_m" + s], out)
            if m > 0:
                fy, fz = D[vec_in + "y_fb_m" + str(m - 1)], D[vec_in + "z_fb_m" + str(m - 1)]
            elif M > 0:
                fy, fz = D["buff_fb_m-1_y"], D["buff_fb_m-1_z"]
            else:
                continue
            self.axpbyz(-1.0j, fz, -1.0, fy, b0)
            self._cdot(b1, "dDHT_minus_m" + s, b0)
            self.append_c2c(out, b1)
            if m < M:
                fy, fz = D[vec_in + "y_fb_m" + str(m + 1)], D[vec_in + "z_fb_m" + str(m + 1)]
                self.axpbyz(-1.0j, fz, 1.0, fy, b0)
                self._cdot(b1, "dDHT_plus_m" + s, b0)
                self.append_c2c(out, b1)

    def field_rot(self, fld_in, fld_out, poisson=False):
        """Spectral curl (transformer_methods_cl.py:185-263): the
        radial-derivative products of every mode and component in one batched
        GEMM, then one combine kernel; with ``poisson`` the 1/w^2 factor of
        field_poiss_vec is applied in the same pass."""
        A, D = self.Args, self.DataDev
        M = A["M"]
        comps = A["vec_comps"]
        G = [D[fld_in + c + "_fb_m" + str(m)] for m in range(M + 1) for c in comps]
        qm, qp = [], []
        for m in range(M + 1):
            for ci in range(3):
                if m > 0:
                    qm.append(("dDHT_minus_m%d" % m, G[3 * (m - 1) + ci]))
                elif M > 0:
                    qm.append(("dDHT_minus_m0", G[3 + ci]))  # G_{+1}, mirrored in the combine
                else:
                    qm.append(None)
                qp.append(("dDHT_plus_m%d" % m, G[3 * (m + 1) + ci]) if m < M else None)
        prods = self._products(qm + qp)
        n = 3 * (M + 1)
        out = [D[fld_out + c + "_fb_m" + str(m)] for m in range(M + 1) for c in comps]
        poiss = PP([self._real_dev("Poiss_m" + str(m)) for m in range(M + 1)]) if poisson else None
        call("ccl_rot_combine", self._dt, M, A["Nr"] - 1, A["Nx"],
             self._real_dev("kx").data_ptr(), PP(G), PP(prods[:n]), PP(prods[n:]), poiss,
             PP(out), stream())
