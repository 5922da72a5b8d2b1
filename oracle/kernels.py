"""THE ORACLE -- test infrastructure only (never imported by the product).

ctypes front ends for the two CPU kernel sets the oracle can run on:

* ``PortKernels``  -- ``oracle/liboracle.so``, this repository's plain-C
  restatement of the reference kernels (``oracle/oracle_kernels.c``).  It
  builds on any host (x86_64 or aarch64).
* ``RefKernels``   -- ``oracle/_ref/libref_*.so``, the reference's own OpenCL
  kernels (``chimeraCL/kernels/*.cl``) compiled unchanged as C++ through
  ``oracle/cl_shim.hpp``.  Only where the reference tree is present.

Both expose the same methods with the same argument meaning, one per reference
kernel (host scalars by value, numpy arrays in place), so ``pic_oracle`` runs
the reference's step on either and the tests can pin one against the other.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_vp = C.c_void_p
_u32 = C.c_uint32
_d = C.c_double
_l = C.c_long
_i = C.c_int
_sz = C.c_size_t


def P(a):
    """Raw data pointer of a C-contiguous numpy array."""
    if a is None:
        return None
    assert a.flags.c_contiguous, "oracle kernels need contiguous arrays"
    return a.ctypes.data_as(_vp)


def _ptrs(arrs):
    arr_t = _vp * len(arrs)
    return arr_t(*[a.ctypes.data for a in arrs])


def _check(a, dtype):
    assert a.dtype == dtype, (a.dtype, dtype)
    assert a.flags.c_contiguous


def build_port(force=False):
    so = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "oracle_kernels.c")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        import subprocess
        base = ["gcc", "-O3", "-fPIC", "-shared", "-ffp-contract=off",
                "-fno-fast-math", "-fno-associative-math"]
        r = subprocess.run(base + ["-fopenmp", "-o", so, src, "-lm"],
                           capture_output=True, text=True)
        if r.returncode != 0:  # a host compiler without OpenMP: serial oracle
            subprocess.run(base + ["-o", so, src, "-lm"], check=True)
    return so


class PortKernels:
    """The oracle's own C restatement of the reference kernels."""

    name = "port"

    def __init__(self):
        self.lib = C.CDLL(build_port())
        L = self.lib
        sig = {
            "port_push_xyz": [_l] + [_vp] * 7 + [_d],
            "port_index_and_sum": [_l] + [_vp] * 5 + [_i, _d, _d, _i, _d, _d],
            "port_sort": [_l] + [_vp] * 4,
            "port_data_align": [_l, _vp, _vp, _vp],
            "port_fill_grid": [_l] + [_vp] * 7 + [_u32] * 4,
            "port_profile_by_interpolant": [_l] + [_vp] * 5 + [_u32],
            "port_depose_scalar": [_i, _u32] + [_vp] * 6 + [_i, _u32, _d, _d, _u32, _d, _d, _vp],
            "port_depose_vector": [_i, _u32] + [_vp] * 10 + [_i, _u32, _d, _d, _u32, _d, _d, _vp],
            "port_gather_and_push": [_i, _l] + [_vp] * 8 + [_d, _u32, _u32, _d, _d, _u32, _d, _d, _vp],
            "port_treat_axis": [_vp, _u32, _i],
            "port_divide_by_dv": [_vp, _u32, _u32, _vp, _i],
            "port_warp_axis": [_vp, _u32, _i],
            "port_profile_edges": [_vp, _vp, _u32, _u32, _u32, _i],
            "port_advance_e_g_m": [_l, _d, _vp, _vp, _vp, _vp],
            "port_get_m1": [_vp, _vp, _u32, _u32],
            "port_get_phase": [_vp, _vp, _d, _u32, _i],
            "port_multiply_by_phase": [_vp, _u32, _u32, _vp],
            "port_append_c2c": [_vp, _vp, _l],
            "port_zpaxz": [_d, _d, _vp, _vp, _l],
            "port_mult_elementwise": [_vp, _vp, _l],
            "port_axpbyz": [_d, _d, _vp, _d, _d, _vp, _vp, _l],
            "port_ab_dot_x": [_d, _d, _vp, _vp, _vp, _u32, _u32],
            "port_cast_c2d": [_vp, _vp, _l],
            "port_num_threads": [],
        }
        for k, v in sig.items():
            getattr(L, k).argtypes = v
            getattr(L, k).restype = _i if k == "port_num_threads" else None

    def num_threads(self):
        return self.lib.port_num_threads()

    # --- particles_generic.cl
    def push_xyz(self, x, y, z, px, py, pz, g_inv, dt):
        self.lib.port_push_xyz(x.size, P(x), P(y), P(z), P(px), P(py), P(pz), P(g_inv), dt)

    def index_and_sum(self, x, y, z, sum_in_cell, indx, Nx, xmin, dx_inv, Nr, rmin, dr_inv):
        _check(sum_in_cell, np.uint32)
        _check(indx, np.uint32)
        self.lib.port_index_and_sum(x.size, P(x), P(y), P(z), P(sum_in_cell), P(indx),
                                    Nx, xmin, dx_inv, Nr, rmin, dr_inv)

    def sort(self, cell_offset, indx, new_sum, sorted_indx):
        self.lib.port_sort(indx.size, P(cell_offset), P(indx), P(new_sum), P(sorted_indx))

    def data_align(self, x, x_new, sorted_indx):
        self.lib.port_data_align(x_new.size, P(x), P(x_new), P(sorted_indx))

    def fill_grid(self, x, y, z, w, theta, xgrid, rgrid, Nx, npx, npr, npth):
        self.lib.port_fill_grid(theta.size, P(x), P(y), P(z), P(w), P(theta), P(xgrid), P(rgrid),
                                Nx, npx, npr, npth)

    def profile_by_interpolant(self, x, w, xx, ff, dxm1):
        self.lib.port_profile_by_interpolant(x.size, P(x), P(w), P(xx), P(ff), P(dxm1), xx.size)

    # --- grid_deposit_m{0,1}.cl (M-generic restatement)
    def depose_scalar(self, M, nxnr_4, sort_indx, x, y, z, w, cell_off, charge,
                      Nx, xmin, dx_inv, Nr, rmin, dr_inv, flds):
        self.lib.port_depose_scalar(M, nxnr_4, P(sort_indx), P(x), P(y), P(z), P(w), P(cell_off),
                                    int(charge), Nx, xmin, dx_inv, Nr, rmin, dr_inv, _ptrs(flds))

    def depose_vector(self, M, nxnr_4, sort_indx, x, y, z, ux, uy, uz, g_inv, w, cell_off,
                      charge, Nx, xmin, dx_inv, Nr, rmin, dr_inv, flds):
        self.lib.port_depose_vector(M, nxnr_4, P(sort_indx), P(x), P(y), P(z), P(ux), P(uy), P(uz),
                                    P(g_inv), P(w), P(cell_off), int(charge), Nx, xmin, dx_inv,
                                    Nr, rmin, dr_inv, _ptrs(flds))

    def gather_and_push(self, M, x, y, z, px, py, pz, g_inv, sort_indx, dt, Np, Np_stay,
                        Nx, xmin, dx_inv, Nr, rmin, dr_inv, flds):
        self.lib.port_gather_and_push(M, Np, P(x), P(y), P(z), P(px), P(py), P(pz), P(g_inv),
                                      P(sort_indx), dt, Np_stay, Nx, xmin, dx_inv, Nr, rmin,
                                      dr_inv, _ptrs(flds))

    # --- grid_generic.cl
    def treat_axis(self, a, Nx):
        self.lib.port_treat_axis(P(a), Nx, 2 if np.iscomplexobj(a) else 1)

    def divide_by_dv(self, a, Nx, dv_inv):
        self.lib.port_divide_by_dv(P(a), a.size, Nx, P(dv_inv), 2 if np.iscomplexobj(a) else 1)

    def warp_axis(self, a, Nx, m):
        self.lib.port_warp_axis(P(a), Nx, m)

    # --- solver_ms_pic.cl
    def profile_edges(self, a, f, Nx, Nf):
        self.lib.port_profile_edges(P(a), P(f), a.size, Nx, Nf, 2 if np.iscomplexobj(a) else 1)

    def advance_e_g_m(self, dt_inv, c1, c2, c3, flds):
        self.lib.port_advance_e_g_m(c1.size, dt_inv, P(c1), P(c2), P(c3), _ptrs(flds))

    # --- transformer_generic.cl
    def get_m1(self, out, inp, Nx):
        self.lib.port_get_m1(P(out), P(inp), Nx, inp.size)

    def get_phase(self, phs, kx, x0, sign):
        self.lib.port_get_phase(P(phs), P(kx), x0, kx.size, sign)

    def multiply_by_phase(self, a, phs):
        self.lib.port_multiply_by_phase(P(a), a.size, phs.size, P(phs))

    # --- generic.cl
    def append_c2c(self, base, add):
        self.lib.port_append_c2c(P(base), P(add), base.size)

    def zpaxz(self, z, a, x):
        self.lib.port_zpaxz(a.real, a.imag, P(x), P(z), x.size)

    def mult_elementwise(self, x, z):
        self.lib.port_mult_elementwise(P(x), P(z), x.size)

    def axpbyz(self, a, x, b, y, z):
        self.lib.port_axpbyz(a.real, a.imag, P(x), b.real, b.imag, P(y), P(z), x.size)

    def ab_dot_x(self, a, b, x, z):
        self.lib.port_ab_dot_x(a.real, a.imag, P(b), P(x), P(z), x.size, b.size)

    def cast_c2d(self, inp, out):
        self.lib.port_cast_c2d(P(inp), P(out), inp.size)


def ref_available():
    d = os.path.join(HERE, "_ref")
    return all(os.path.exists(os.path.join(d, f"libref_{n}.so"))
               for n in ("common", "grid_m0", "grid_m1"))


class RefKernels:
    """The reference's own OpenCL kernels, compiled unchanged as C++ (serial).

    Launch sizes follow the reference's methods layer: deposits run the four
    colour offsets over NxNr_4 work-items each (grid_methods_cl.py:44-95),
    everything else one work-item per element."""

    name = "ref"

    def __init__(self):
        if not ref_available():
            raise RuntimeError("oracle/_ref is not built (make -C oracle ref)")
        d = os.path.join(HERE, "_ref")
        self.c = C.CDLL(os.path.join(d, "libref_common.so"))
        self.g = {0: C.CDLL(os.path.join(d, "libref_grid_m0.so")),
                  1: C.CDLL(os.path.join(d, "libref_grid_m1.so"))}
        c = self.c
        sig = {
            "ref_set_cdouble_to": [_sz, _vp, _d, _d, _u32],
            "ref_append_c2c": [_sz, _vp, _vp, _u32],
            "ref_zpaxz_c2c": [_sz, _d, _d, _vp, _vp, _u32],
            "ref_mult_elementwise_d2c": [_sz, _vp, _vp, _u32],
            "ref_axpbyz_c2c": [_sz, _d, _d, _vp, _d, _d, _vp, _vp, _u32],
            "ref_ab_dot_x": [_sz, _d, _d, _vp, _vp, _vp, _u32, _u32],
            "ref_cast_array_d2c": [_sz, _vp, _vp, _u32],
            "ref_divide_by_dv_d": [_sz, _vp, _u32, _u32, _vp],
            "ref_divide_by_dv_c": [_sz, _vp, _u32, _u32, _vp],
            "ref_treat_axis_d": [_sz, _vp, _u32],
            "ref_treat_axis_c": [_sz, _vp, _u32],
            "ref_warp_axis_m0_d": [_sz, _vp, _u32],
            "ref_warp_axis_m1plus_c": [_sz, _vp, _u32],
            "ref_profile_by_interpolant": [_sz, _vp, _vp, _u32, _vp, _vp, _vp, _u32],
            "ref_fill_grid": [_sz] + [_vp] * 7 + [_u32] * 5,
            "ref_index_and_sum_in_cell": [_sz, _vp, _vp, _vp, _vp, _u32, _vp, _u32, _d, _d, _u32, _d, _d],
            "ref_push_xyz": [_sz] + [_vp] * 7 + [_d, _u32],
            "ref_data_align_dbl": [_sz, _vp, _vp, _vp, _u32],
            "ref_sort": [_sz, _vp, _vp, _vp, _vp, _u32],
            "ref_profile_edges_c": [_sz, _vp, _vp, _u32, _u32, _u32],
            "ref_profile_edges_d": [_sz, _vp, _vp, _u32, _u32, _u32],
            "ref_advance_e_g_m": [_sz, _u32, _d, _vp, _vp, _vp, _vp],
            "ref_get_m1": [_sz, _vp, _vp, _u32, _u32],
            "ref_get_phase_plus": [_sz, _vp, _vp, _d, _u32],
            "ref_get_phase_minus": [_sz, _vp, _vp, _d, _u32],
            "ref_multiply_by_phase": [_sz, _vp, _u32, _u32, _vp],
        }
        for k, v in sig.items():
            getattr(c, k).argtypes = v
            getattr(c, k).restype = None
        for g in self.g.values():
            g.ref_depose_scalar.argtypes = [_sz, _u32] + [_vp] * 6 + [_i, _u32, _d, _d, _u32, _d, _d, _u32, _vp]
            g.ref_depose_vector.argtypes = [_sz, _u32] + [_vp] * 10 + [_i, _u32, _d, _d, _u32, _d, _d, _u32, _vp]
            g.ref_gather_and_push.argtypes = [_sz] + [_vp] * 9 + [_d, _u32, _u32, _u32, _d, _d, _u32, _d, _d, _u32, _vp]
            for f in (g.ref_depose_scalar, g.ref_depose_vector, g.ref_gather_and_push):
                f.restype = None

    def _grid(self, M):
        if M not in self.g:
            raise NotImplementedError("the reference ships deposit kernels for M<=1 only")
        return self.g[M]

    def push_xyz(self, x, y, z, px, py, pz, g_inv, dt):
        self.c.ref_push_xyz(x.size, P(x), P(y), P(z), P(px), P(py), P(pz), P(g_inv), dt, x.size)

    def index_and_sum(self, x, y, z, sum_in_cell, indx, Nx, xmin, dx_inv, Nr, rmin, dr_inv):
        self.c.ref_index_and_sum_in_cell(x.size, P(x), P(y), P(z), P(sum_in_cell), x.size, P(indx),
                                         Nx, xmin, dx_inv, Nr, rmin, dr_inv)

    def sort(self, cell_offset, indx, new_sum, sorted_indx):
        self.c.ref_sort(indx.size, P(cell_offset), P(indx), P(new_sum), P(sorted_indx), indx.size)

    def data_align(self, x, x_new, sorted_indx):
        self.c.ref_data_align_dbl(x_new.size, P(x), P(x_new), P(sorted_indx), x_new.size)

    def fill_grid(self, x, y, z, w, theta, xgrid, rgrid, Nx, npx, npr, npth):
        self.c.ref_fill_grid(theta.size, P(x), P(y), P(z), P(w), P(theta), P(xgrid), P(rgrid),
                             Nx, theta.size, npx, npr, npth)

    def profile_by_interpolant(self, x, w, xx, ff, dxm1):
        self.c.ref_profile_by_interpolant(x.size, P(x), P(w), x.size, P(xx), P(ff), P(dxm1), xx.size)

    def depose_scalar(self, M, nxnr_4, sort_indx, x, y, z, w, cell_off, charge,
                      Nx, xmin, dx_inv, Nr, rmin, dr_inv, flds):
        g = self._grid(M)
        for off in range(4):
            g.ref_depose_scalar(nxnr_4, off, P(sort_indx), P(x), P(y), P(z), P(w), P(cell_off),
                                int(charge), Nx, xmin, dx_inv, Nr, rmin, dr_inv, nxnr_4, _ptrs(flds))

    def depose_vector(self, M, nxnr_4, sort_indx, x, y, z, ux, uy, uz, g_inv, w, cell_off,
                      charge, Nx, xmin, dx_inv, Nr, rmin, dr_inv, flds):
        g = self._grid(M)
        for off in range(4):
            g.ref_depose_vector(nxnr_4, off, P(sort_indx), P(x), P(y), P(z), P(ux), P(uy), P(uz),
                                P(g_inv), P(w), P(cell_off), int(charge), Nx, xmin, dx_inv, Nr,
                                rmin, dr_inv, nxnr_4, _ptrs(flds))

    def gather_and_push(self, M, x, y, z, px, py, pz, g_inv, sort_indx, dt, Np, Np_stay,
                        Nx, xmin, dx_inv, Nr, rmin, dr_inv, flds):
        g = self._grid(M)
        # cell_offset is an argument the reference kernel never reads
        dummy = np.zeros(1, np.uint32)
        g.ref_gather_and_push(Np, P(x), P(y), P(z), P(px), P(py), P(pz), P(g_inv), P(sort_indx),
                              P(dummy), dt, Np, Np_stay, Nx, xmin, dx_inv, Nr, rmin, dr_inv,
                              (Nx - 1) * (Nr - 1), _ptrs(flds))

    def treat_axis(self, a, Nx):
        (self.c.ref_treat_axis_c if np.iscomplexobj(a) else self.c.ref_treat_axis_d)(Nx, P(a), Nx)

    def divide_by_dv(self, a, Nx, dv_inv):
        f = self.c.ref_divide_by_dv_c if np.iscomplexobj(a) else self.c.ref_divide_by_dv_d
        f(a.size, P(a), a.size, Nx, P(dv_inv))

    def warp_axis(self, a, Nx, m):
        (self.c.ref_warp_axis_m0_d if m == 0 else self.c.ref_warp_axis_m1plus_c)(Nx, P(a), Nx)

    def profile_edges(self, a, f, Nx, Nf):
        g = self.c.ref_profile_edges_c if np.iscomplexobj(a) else self.c.ref_profile_edges_d
        g(a.size, P(a), P(f), a.size, Nx, Nf)

    def advance_e_g_m(self, dt_inv, c1, c2, c3, flds):
        self.c.ref_advance_e_g_m(c1.size, c1.size, dt_inv, P(c1), P(c2), P(c3), _ptrs(flds))

    def get_m1(self, out, inp, Nx):
        self.c.ref_get_m1(inp.size, P(out), P(inp), Nx, inp.size)

    def get_phase(self, phs, kx, x0, sign):
        f = self.c.ref_get_phase_plus if sign > 0 else self.c.ref_get_phase_minus
        f(kx.size, P(phs), P(kx), x0, kx.size)

    def multiply_by_phase(self, a, phs):
        self.c.ref_multiply_by_phase(a.size, P(a), a.size, phs.size, P(phs))

    def append_c2c(self, base, add):
        self.c.ref_append_c2c(base.size, P(base), P(add), base.size)

    def zpaxz(self, z, a, x):
        self.c.ref_zpaxz_c2c(x.size, a.real, a.imag, P(x), P(z), x.size)

    def mult_elementwise(self, x, z):
        self.c.ref_mult_elementwise_d2c(x.size, P(x), P(z), x.size)

    def axpbyz(self, a, x, b, y, z):
        self.c.ref_axpbyz_c2c(x.size, a.real, a.imag, P(x), b.real, b.imag, P(y), P(z), x.size)

    def ab_dot_x(self, a, b, x, z):
        self.c.ref_ab_dot_x(x.size, a.real, a.imag, P(b), P(x), P(z), x.size, b.size)

    def cast_c2d(self, inp, out):
        self.c.ref_cast_array_d2c(inp.size, P(inp), P(out), inp.size)


def get_kernels(kind="port"):
    return RefKernels() if kind == "ref" else PortKernels()
