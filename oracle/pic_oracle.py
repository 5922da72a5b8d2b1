"""THE ORACLE -- test infrastructure only (never imported by the product).

A CPU restatement of chimeraCL's quasi-cylindrical PSATD PIC step, host side:
the reference's wrapper classes and ``methods/*.py`` call sequence, on numpy
arrays, with every reference OpenCL kernel executed by one of the two CPU kernel
sets of ``oracle.kernels`` (the repository's C restatement, or the reference's
own kernels compiled unchanged).  The third-party arithmetic on the path is
restated with the reference's own CPU stand-ins: ``numpy.fft`` (forward
unnormalised, inverse normalised, as Reikna FFT / pyFFTW,
transformer_methods_cl.py:482-509) and ``numpy.dot`` for the Hankel transforms
(the reference's CPU path, transformer_methods_cl.py:474-480); scipy
``jn_zeros``/``jn`` and ``numpy.linalg.pinv`` build the matrices exactly as
transformer.py:65-97 does.

The only input the reference draws from a random generator, the per-cell theta
jitter of a new plasma domain (particles_methods_cl.py:85-87, Threefry there),
comes here from ``numpy.random.Generator(PCG64(seed))`` -- the same stream the
product draws, so both sides start from identical particles.  Threefry itself
is not restated (parity unpinned for the generator, by design).
"""
import copy

import numpy as np
from scipy.special import jn, jn_zeros

from .kernels import get_kernels

# The longitudinal transforms: numpy's FFT by default (forward unnormalised,
# inverse 1/N, the convention of the reference's pyFFTW/numpy path).  The
# timed CPU baseline may switch to scipy's multi-threaded FFT of the same
# convention (use_threaded_fft); the tests and fixtures keep numpy's.
_FFT = {"fft": np.fft.fft, "ifft": np.fft.ifft}


def use_threaded_fft(workers=-1):
    """Take scipy.fft with `workers` threads for the oracle's transforms
    (same convention; results differ from numpy's in the last bits)."""
    import scipy.fft as sf
    _FFT["fft"] = lambda a, axis: sf.fft(a, axis=axis, workers=workers)
    _FFT["ifft"] = lambda a, axis: sf.ifft(a, axis=axis, workers=workers)


def use_numpy_fft():
    _FFT["fft"], _FFT["ifft"] = np.fft.fft, np.fft.ifft

VEC = ("x", "y", "z")


def make_rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


# ----------------------------------------------------------------------
class OGrid:
    """Grid + Transformer + Solver state (grid.py, transformer.py, solver.py)."""

    def __init__(self, cfg, K=None, solver=True):
        self.K = K or get_kernels("port")
        self.Args = A = cfg
        # grid.py:68-103
        A.setdefault("M", 0)
        A["dx"] = (A["Xmax"] - A["Xmin"]) / (A["Nx"] - 1)
        A["dx_inv"] = 1.0 / A["dx"]
        A["dr"] = A["Rmax"] / (A["Nr"] - 1.5)
        A["dr_inv"] = 1.0 / A["dr"]
        if "dt" not in A:
            A["dt"] = A["dx"]
        A["dt_inv"] = 1.0 / A["dt"]
        A["Xgrid"] = A["Xmin"] + A["dx"] * np.arange(A["Nx"])
        A["Rmin"] = -0.5 * A["dr"]
        A["Rgrid"] = A["Rmin"] + A["dr"] * np.arange(A["Nr"])
        A["Rmax"] = A["Rgrid"].max()
        with np.errstate(divide="ignore"):
            A["dV_inv"] = (A["Rgrid"] > 0) / (2 * np.pi * A["dx"] * A["dr"] * A["Rgrid"])
        A["NxNr"] = A["Nr"] * A["Nx"]
        A["Nxm1Nrm1"] = (A["Nr"] - 1) * (A["Nx"] - 1)
        A["NxNrm1"] = (A["Nr"] - 1) * A["Nx"]
        A["NxNr_4"] = (A["Nr"]) // 2 * (A["Nx"]) // 2
        A["vec_comps"] = list(VEC)
        M, Nx, Nr = A["M"], A["Nx"], A["Nr"]
        self.D = D = {}
        for f in ("E", "B", "J", "G", "rho"):
            comps = [f + c for c in VEC] if f != "rho" else ["rho"]
            for fc in comps:
                D[fc + "_m0"] = np.zeros((Nr, Nx))
                for m in range(1, M + 1):
                    D[fc + "_m" + str(m)] = np.zeros((Nr, Nx), np.complex128)
        if solver:
            self._init_solver()

    # solver_methods_cl.py:32-41
    def _init_damping(self):
        N = int(self.Args["DampCells"])
        z = np.arange(2 * N)
        z_shft = 3.0 * (z - N + 1) / (N + 1)
        self.Args["DampProfile"] = ((z < 4.0 * N / 3) * (z >= N) * np.sin(0.5 * np.pi * z_shft) ** 2
                                    + (z >= 4.0 * N / 3)).astype(np.float64)

    def _init_solver(self):
        A, D = self.Args, self.D
        M, Nx, Nr = A["M"], A["Nx"], A["Nr"]
        if "DampCells" in A:
            self._init_damping()
        for f in ("E", "B", "G", "J", "dN0", "dN1"):
            for c in VEC:
                for m in range(M + 1):
                    D[f + c + "_fb_m" + str(m)] = np.zeros((Nr - 1, Nx), np.complex128)
        for m in range(M + 1):
            D["rho_fb_m" + str(m)] = np.zeros((Nr - 1, Nx), np.complex128)
        for c in VEC:
            D["buff_fb_m-1_" + c] = np.zeros((Nr - 1, Nx), np.complex128)
        # transformer.py:28-63
        dx, dr = A["dx"], A["dr"]
        kx = 2 * np.pi * np.fft.fftfreq(Nx, dx)
        R_period = A["Rgrid"][-1] + 0.5 * dr
        A["kx"] = kx
        for m in range(M + 2):
            A["kr_m" + str(m)] = jn_zeros(m, Nr - 1) / R_period
        for m in range(M + 1):
            kr = A["kr_m" + str(m)]
            A["w_m" + str(m)] = np.sqrt(kx[None, :] ** 2 + kr[:, None] ** 2)
            A["Poiss_m" + str(m)] = 1.0 / A["w_m" + str(m)] ** 2
            A["SmoothingFilter_m" + str(m)] = (
                (1 - np.sin(0.5 * np.pi * kx[None, :] / kx.max()) ** 2)
                * (1 - np.sin(0.5 * np.pi * kr[:, None] / kr.max()) ** 2))
        # transformer.py:65-97
        Rg = A["Rgrid"][1:, None]
        Rp = Rg[-1] + 0.5 * dr
        for m in range(M + 1):
            kr0 = jn_zeros(m, Nr - 1) / Rp
            krp = jn_zeros(m + 1, Nr - 1) / Rp
            krm = jn_zeros(m - 1, Nr - 1) / Rp
            A["DHT_inv_m" + str(m)] = jn(m, Rg * kr0)
            A["DHT_m" + str(m)] = np.linalg.pinv(A["DHT_inv_m" + str(m)])
            A["dDHT_plus_m" + str(m)] = A["DHT_m" + str(m)].dot(0.5 * krp * jn(m, Rg * krp))
            A["dDHT_minus_m" + str(m)] = A["DHT_m" + str(m)].dot(0.5 * krm * jn(m, Rg * krm))
        # solver.py:41-52
        for m in range(M + 1):
            w = A["w_m" + str(m)]
            dt = A["dt"]
            A["MxSlv_cos(wdt)_m" + str(m)] = np.cos(w * dt)
            A["MxSlv_sin(wdt)*w_m" + str(m)] = np.sin(w * dt) * w
            A["MxSlv_1/w**2_m" + str(m)] = 1.0 / w ** 2
        self.phs = np.zeros(Nx, np.complex128)

    # ---------------- grid.py:23-66 + grid_methods_cl.py
    def depose_charge(self, species=()):
        A, D, K = self.Args, self.D, self.K
        for m in range(A["M"] + 1):
            D["rho_m" + str(m)][:] = 0
        for p in species:
            if p.Args["Np"] <= 0:
                continue
            flds = [D["rho_m" + str(m)] for m in range(A["M"] + 1)]
            K.depose_scalar(A["M"], A["NxNr_4"], p.D["sort_indx"], p.D["x"], p.D["y"], p.D["z"],
                            p.D["w"], p.D["cell_offset"], np.int8(p.Args["charge"]), A["Nx"],
                            A["Xmin"], A["dx_inv"], A["Nr"], A["Rmin"], A["dr_inv"], flds)
        self._postproc(["rho"])

    def depose_currents(self, species=()):
        A, D, K = self.Args, self.D, self.K
        M = A["M"]
        for m in range(M + 1):
            for c in VEC:
                D["J" + c + "_m" + str(m)][:] = 0
        for p in species:
            if "Immobile" in p.Args:
                continue
            flds = [D["J" + c + "_m" + str(m)] for m in range(M + 1) for c in VEC]
            K.depose_vector(M, A["NxNr_4"], p.D["sort_indx"], p.D["x"], p.D["y"], p.D["z"],
                            p.D["px"], p.D["py"], p.D["pz"], p.D["g_inv"], p.D["w"],
                            p.D["cell_offset"], np.int8(p.Args["charge"]), A["Nx"], A["Xmin"],
                            A["dx_inv"], A["Nr"], A["Rmin"], A["dr_inv"], flds)
        self._postproc(["J" + c for c in VEC])

    def _postproc(self, names):
        # grid_methods_cl.py:98-151: axis row, then 1/dV, per component
        A, D, K = self.Args, self.D, self.K
        for f in names:
            arrs = [D[f + "_m" + str(m)] for m in range(A["M"] + 1)]
            for a in arrs:
                K.treat_axis(a, A["Nx"])
            for a in arrs:
                K.divide_by_dv(a, A["Nx"], A["dV_inv"])

    def gather_and_push(self, species=()):
        A, D, K = self.Args, self.D, self.K
        M = A["M"]
        for f in ("E", "B"):
            for c in VEC:
                for m in range(M + 1):
                    K.warp_axis(D[f + c + "_m" + str(m)], A["Nx"], m)
        for p in species:
            if "Immobile" in p.Args:
                continue
            flds = [D[f + c + "_m" + str(m)] for m in range(M + 1) for f in ("E", "B") for c in VEC]
            K.gather_and_push(M, p.D["x"], p.D["y"], p.D["z"], p.D["px"], p.D["py"], p.D["pz"],
                              p.D["g_inv"], p.D["sort_indx"], p.Args["FactorPush"], p.Args["Np"],
                              p.Args["Np_stay"], A["Nx"], A["Xmin"], A["dx_inv"], A["Nr"],
                              A["Rmin"], A["dr_inv"], flds)

    # ---------------- transformer.py:17-26 + transformer_methods_cl.py
    def fb_transform(self, scals=(), vects=(), dir=0, mode="full"):
        for s in scals:
            self.transform_field(s, dir, mode)
        for v in vects:
            for c in VEC:
                self.transform_field(v + c, dir, mode)

    def transform_field(self, arg, dir, mode):
        A, D, K = self.Args, self.D, self.K
        M = A["M"]
        K.get_phase(self.phs, A["kx"], A["Xmin"], +1 if dir == 1 else -1)
        phs = self.phs
        for m in range(M + 1):
            s = str(m)
            if dir == 0:
                src = D[arg + "_m" + s][1:]
                if mode == "full":
                    if m == 0:
                        out = np.dot(A["DHT_m0"], np.ascontiguousarray(src)).astype(np.complex128)
                    else:
                        out = np.dot(A["DHT_m" + s], np.ascontiguousarray(src))
                else:
                    out = src.astype(np.complex128)
                out = np.ascontiguousarray(_FFT["fft"](out, axis=1))
                K.multiply_by_phase(out, phs)
                D[arg + "_fb_m" + s][:] = out
            else:
                buf = D[arg + "_fb_m" + s].copy()
                K.multiply_by_phase(buf, phs)
                buf = np.ascontiguousarray(_FFT["ifft"](buf, axis=1))
                if m == 0:
                    re = np.empty(buf.shape)
                    K.cast_c2d(buf, re)
                    buf = re
                if mode == "full":
                    buf = np.dot(A["DHT_inv_m" + s], buf)
                D[arg + "_m" + s][1:] = buf

    def fields_smooth(self, flds):
        A, D, K = self.Args, self.D, self.K
        for m in range(A["M"] + 1):
            for f in flds:
                K.mult_elementwise(A["SmoothingFilter_m" + str(m)], D[f + "_fb_m" + str(m)])

    def field_poiss_vec(self, fld):
        A, D, K = self.Args, self.D, self.K
        for m in range(A["M"] + 1):
            for c in VEC:
                K.mult_elementwise(A["Poiss_m" + str(m)], D[fld + c + "_fb_m" + str(m)])

    def _get_mm1(self, fld, comp):
        if self.Args["M"] == 0:
            return
        self.K.get_m1(self.D["buff_fb_m-1_" + comp], self.D[fld + "_fb_m1"], self.Args["Nx"])

    def _cdot(self, A_, X):
        return np.ascontiguousarray(np.dot(A_, X))

    def field_grad(self, scl_in, vec_out):
        A, D, K = self.Args, self.D, self.K
        M = A["M"]
        self._get_mm1(scl_in, "x")
        for m in range(M + 1):
            s = str(m)
            ox, oy, oz = (D[vec_out + c + "_fb_m" + s] for c in VEC)
            for o in (ox, oy, oz):
                o[:] = 0
            K.ab_dot_x(1j, A["kx"], D[scl_in + "_fb_m" + s], ox)
            if m > 0:
                f = D[scl_in + "_fb_m" + str(m - 1)]
            elif M > 0:
                f = D["buff_fb_m-1_x"]
            else:
                continue
            b = self._cdot(A["dDHT_minus_m" + s], f)
            K.zpaxz(oy, complex(-1.0), b)
            K.zpaxz(oz, complex(-1j), b)
            if m < M:
                b = self._cdot(A["dDHT_plus_m" + s], D[scl_in + "_fb_m" + str(m + 1)])
                K.append_c2c(oy, b)
                K.zpaxz(oz, complex(-1j), b)

    def field_div(self, vin, sout):
        """transformer_methods_cl.py:135-183: i kx V_x plus the radial
        derivative products of (-i V_z - V_y) of mode m-1 (the m=-1 mirror
        for m = 0) and of (-i V_z + V_y) of mode m+1."""
        A, D, K = self.Args, self.D, self.K
        M = A["M"]
        for c in ("y", "z"):
            self._get_mm1(vin + c, c)
        for m in range(M + 1):
            s = str(m)
            out = D[sout + "_fb_m" + s]
            out[:] = 0
            K.ab_dot_x(1j, A["kx"], D[vin + "x_fb_m" + s], out)
            if m > 0:
                fy, fz = D[vin + "y_fb_m" + str(m - 1)], D[vin + "z_fb_m" + str(m - 1)]
            elif M > 0:
                fy, fz = D["buff_fb_m-1_y"], D["buff_fb_m-1_z"]
            else:
                continue
            b0 = np.zeros_like(out)
            K.axpbyz(-1j, fz, -1.0, fy, b0)
            K.append_c2c(out, self._cdot(A["dDHT_minus_m" + s], b0))
            if m < M:
                fy, fz = D[vin + "y_fb_m" + str(m + 1)], D[vin + "z_fb_m" + str(m + 1)]
                K.axpbyz(-1j, fz, 1.0, fy, b0)
                K.append_c2c(out, self._cdot(A["dDHT_plus_m" + s], b0))

    def field_rot(self, fin, fout):
        A, D, K = self.Args, self.D, self.K
        M = A["M"]
        for c in VEC:
            self._get_mm1(fin + c, c)
        b0 = np.zeros((A["Nr"] - 1, A["Nx"]), np.complex128)
        for m in range(M + 1):
            s = str(m)
            ox, oy, oz = (D[fout + c + "_fb_m" + s] for c in VEC)
            for o in (ox, oy, oz):
                o[:] = 0
            K.ab_dot_x(-1j, A["kx"], D[fin + "z_fb_m" + s], oy)
            K.ab_dot_x(1j, A["kx"], D[fin + "y_fb_m" + s], oz)
            if m > 0:
                fx, fy, fz = (D[fin + c + "_fb_m" + str(m - 1)] for c in VEC)
            elif M > 0:
                fx, fy, fz = (D["buff_fb_m-1_" + c] for c in VEC)
            else:
                continue
            K.axpbyz(complex(-1), fz, complex(1j), fy, b0)
            K.append_c2c(ox, self._cdot(A["dDHT_minus_m" + s], b0))
            b = self._cdot(A["dDHT_minus_m" + s], fx)
            K.zpaxz(oy, complex(-1j), b)
            K.zpaxz(oz, complex(1), b)
            if m < M:
                fx, fy, fz = (D[fin + c + "_fb_m" + str(m + 1)] for c in VEC)
                K.axpbyz(complex(1), fz, complex(1j), fy, b0)
                K.append_c2c(ox, self._cdot(A["dDHT_plus_m" + s], b0))
                b = self._cdot(A["dDHT_plus_m" + s], fx)
                K.zpaxz(oy, complex(-1j), b)
                K.zpaxz(oz, complex(-1), b)

    # ---------------- solver.py:29-39 + solver_methods_cl.py
    def push_fields(self):
        A, D, K = self.Args, self.D, self.K
        for m in range(A["M"] + 1):
            s = str(m)
            flds = [D[v + c + "_fb_m" + s] for v in ("E", "G", "J", "dN0", "dN1") for c in VEC]
            K.advance_e_g_m(A["dt_inv"], A["MxSlv_cos(wdt)_m" + s], A["MxSlv_sin(wdt)*w_m" + s],
                            A["MxSlv_1/w**2_m" + s], flds)

    def profile_edges(self, flds):
        A, D, K = self.Args, self.D, self.K
        for f in flds:
            for c in VEC:
                for m in range(A["M"] + 1):
                    K.profile_edges(D[f + c + "_m" + str(m)], A["DampProfile"], A["Nx"],
                                    2 * int(A["DampCells"]))

    def damp_fields(self):
        self.fb_transform(vects=["E", "G"], dir=1, mode="half")
        self.profile_edges(["E", "G"])
        self.fb_transform(vects=["E", "G"], dir=0, mode="half")

    def restore_B_fb(self):
        self.field_rot("G", "B")
        self.field_poiss_vec("B")


# ----------------------------------------------------------------------
class OSpecies:
    """Particles (particles.py + particles_methods_cl.py)."""

    def __init__(self, cfg, K=None, seed=0):
        self.K = K or get_kernels("port")
        self.rng = make_rng(seed)
        self.Args = A = cfg
        A["Np"] = 0
        A["Np_stay"] = 0
        A.setdefault("dt", 1.0)
        A.setdefault("dx", 1.0)
        A.setdefault("dr", 1.0)
        A.setdefault("charge", -1.0)
        A.setdefault("mass", 1.0)
        A.setdefault("dens", 1.0)
        dt, q, ms, n, dx, dr = (A[k] for k in ("dt", "charge", "mass", "dens", "dx", "dr"))
        A["dt_2"] = 0.5 * dt
        if "Nppc" in A:
            A["Nppc"] = np.array(A["Nppc"], dtype=np.uint32)
            A["w0"] = 2 * np.pi * dx * dr * n / np.prod(A["Nppc"])
            A["ddx"] = dx / A["Nppc"][0]
        else:
            A["ddx"] = 1.0
        A["FactorPush"] = 2 * np.pi * dt * q / ms
        A["right_lim"] = 0.0
        self.flag_sorted = False
        comps = self.comps()
        self.D = {k: np.zeros(0) for k in comps}

    def comps(self):
        if "Immobile" in self.Args:
            return ["x", "y", "z", "w"]
        return ["x", "y", "z", "px", "py", "pz", "w", "g_inv"]

    def reset_num_parts(self):
        Np = self.D["x"].size
        self.Args["Np"] = Np
        self.Args["Np_stay"] = Np

    def add_new_particles(self, source=None):
        src = self.D if source is None else source.D
        for a in self.comps():
            self.D[a] = np.concatenate([self.D[a], src[a + "_new"]])
        self.reset_num_parts()
        self.flag_sorted = False

    def add_particles(self, domain_in=None, source=None, density_profiles=None):
        if source is None:
            self.make_new_domain(domain_in, density_profiles=density_profiles)
            self.add_new_particles()
        else:
            self.add_new_particles(source=source)

    def make_new_domain(self, pin, density_profiles=None):
        A, D, K = self.Args, self.D, self.K
        xmin, xmax, rmin, rmax = (pin[k] for k in ("Xmin", "Xmax", "Rmin", "Rmax"))
        Nx_loc = int(np.ceil((xmax - xmin) / A["dx"]) + 1)
        Nr_loc = int(np.round((rmax - rmin) / A["dr"]) + 1)
        Xg = xmin + A["dx"] * np.arange(Nx_loc)
        Rg = rmin + A["dr"] * np.arange(Nr_loc)
        A["right_lim"] = Xg[-1]
        nc = (Nx_loc - 1) * (Nr_loc - 1)
        Np = int(nc * np.prod(A["Nppc"]))
        for a in ("x", "y", "z", "w"):
            D[a + "_new"] = np.empty(Np)
        theta = 0.0 + (2 * np.pi - 0.0) * self.rng.random(nc)
        npx, npr, npth = (int(v) for v in A["Nppc"])
        K.fill_grid(D["x_new"], D["y_new"], D["z_new"], D["w_new"], theta, Xg, Rg, Nx_loc,
                    npx, npr, npth)
        D["w_new"] *= A["w0"]
        if density_profiles is not None:
            for prf in density_profiles:
                if prf["coord"] != "x":
                    continue
                self.dens_profile(prf["points"], prf["values"], pin["Xmin"], pin["Xmax"],
                                  coord=prf["coord"] + "_new", weight="w_new")
        if "Immobile" not in A:
            for a in ("px", "py", "pz"):
                if "d" + a not in pin and a + "_c" not in pin:
                    D[a + "_new"] = np.zeros(Np)
                    pin[a + "_c"] = 0
                    pin["d" + a] = 0
                else:
                    pin.setdefault(a + "_c", 0)
                    if "d" + a in pin:
                        D[a + "_new"] = pin[a + "_c"] + pin["d" + a] * self.rng.standard_normal(Np)
                    else:
                        pin["d" + a] = 0
                        D[a + "_new"] = np.full(Np, float(pin[a + "_c"]))
            mom = sum(pin[k] ** 2 for k in ("px_c", "py_c", "pz_c", "dpx", "dpy", "dpz"))
            if mom != 0:
                D["g_inv_new"] = 1.0 / np.sqrt(1 + D["px_new"] * D["px_new"] + D["py_new"]
                                               * D["py_new"] + D["pz_new"] * D["pz_new"])
            else:
                D["g_inv_new"] = np.ones(Np)

    def make_new_beam(self, pin):
        """particles_methods_cl.py:149-177; normal draws from the seeded
        PCG64 stream in the order x, y, z, px, py, pz."""
        D, Np = self.D, int(pin["Np"])
        for a in ("x", "y", "z"):
            D[a + "_new"] = pin[a + "_c"] + pin["L" + a] * self.rng.standard_normal(Np)
        for a in ("px", "py", "pz"):
            pin.setdefault(a + "_c", 0)
            pin.setdefault("d" + a, 0)
            D[a + "_new"] = pin[a + "_c"] + pin["d" + a] * self.rng.standard_normal(Np)
        D["w_new"] = np.full(Np, pin["FullCharge"] / pin["Np"])
        D["g_inv_new"] = 1.0 / np.sqrt(1 + D["px_new"] * D["px_new"] + D["py_new"] * D["py_new"]
                                       + D["pz_new"] * D["pz_new"])

    def dens_profile(self, x_prf, f_prf, xmin, xmax, coord="x", weight="w"):
        x_prf = np.array(x_prf, dtype=np.double)
        f_prf = np.array(f_prf, dtype=np.double)
        i0 = (x_prf < xmin).sum() - 1
        i1 = (x_prf < xmax).sum() + 1
        xl = np.ascontiguousarray(x_prf[i0:i1])
        fl = np.ascontiguousarray(f_prf[i0:i1])
        dxm1 = 1.0 / (xl[1:] - xl[:-1])
        self.K.profile_by_interpolant(self.D[coord], self.D[weight], xl, fl, dxm1)

    def push_coords(self, mode="half"):
        A, D = self.Args, self.D
        if A["Np"] == 0 or "Immobile" in A:
            return
        dt = A["dt_2"] if mode == "half" else A["dt"]
        self.K.push_xyz(D["x"], D["y"], D["z"], D["px"], D["py"], D["pz"], D["g_inv"], dt)
        self.flag_sorted = False

    def sort_parts(self, grid):
        if self.Args["Np"] == 0:
            self.flag_sorted = True
        if not self.flag_sorted:
            self.index_sort(grid)
            self.flag_sorted = True

    def index_sort(self, grid):
        A, D, K, G = self.Args, self.D, self.K, grid.Args
        Np = A["Np"]
        D["indx_in_cell"] = np.empty(Np, np.uint32)
        D["sum_in_cell"] = np.zeros(G["Nxm1Nrm1"] + 1, np.uint32)
        K.index_and_sum(D["x"], D["y"], D["z"], D["sum_in_cell"], D["indx_in_cell"], G["Nx"],
                        G["Xmin"], G["dx_inv"], G["Nr"], G["Rmin"], G["dr_inv"])
        co = np.zeros(D["sum_in_cell"].size + 1, np.uint32)
        co[1:] = np.cumsum(D["sum_in_cell"].astype(np.int64)).astype(np.uint32)
        D["cell_offset"] = co
        D["sum_in_cell"][:] = 0
        A["Np_stay"] = int(co[-2])
        D["sort_indx"] = np.empty(Np, np.uint32)
        K.sort(co, D["indx_in_cell"], D["sum_in_cell"], D["sort_indx"])

    def align_parts(self):
        if self.Args["Np"] == 0:
            return
        comps = self.comps()
        A, D = self.Args, self.D
        ns = A["Np_stay"]
        if ns == 0:
            for c in comps + ["sort_indx"]:
                D[c] = np.zeros(0, D[c].dtype)
            self.reset_num_parts()
            return
        for c in comps:
            buf = np.empty(ns, D[c].dtype)
            self.K.data_align(D[c], buf, D["sort_indx"])
            D[c] = buf
        D["sort_indx"] = np.arange(ns, dtype=np.uint32)
        self.reset_num_parts()

    def free_added(self):
        for a in self.comps():
            self.D.pop(a + "_new", None)


# ----------------------------------------------------------------------
class OFrame:
    """Moving window (frame.py)."""

    def __init__(self, cfg):
        self.Args = A = cfg
        A.setdefault("Steps", 1.0)
        A.setdefault("Velocity", 0.0)
        A.setdefault("dt", 1)
        A.setdefault("DensityProfiles", None)

    def shift_grids(self, grids=(), steps=None):
        steps = self.Args["Steps"] if steps is None else steps
        sh = steps * self.Args["dt"] * self.Args["Velocity"]
        for g in grids:
            for k in ("Xmax", "Xmin", "Xgrid"):
                g.Args[k] += sh

    def inject_plasma(self, species, grid, steps=None):
        steps = self.Args["Steps"] if steps is None else steps
        sh = steps * self.Args["dt"] * self.Args["Velocity"]
        for sp in species:
            if sp.Args["Np"] == 0:
                sp.Args["right_lim"] = grid.Args["Xmax"] - sh
            dom = {"Xmin": sp.Args["right_lim"]}
            dom["Xmax"] = dom["Xmin"] + sh
            dom["Rmin"] = grid.Args["Rmin"] * (grid.Args["Rmin"] > 0)
            dom["Rmax"] = grid.Args["Rmax"]
            sp.make_new_domain(dom, density_profiles=self.Args["DensityProfiles"])
            if "InjectorSource" in sp.Args:
                sp.add_new_particles(sp.Args["InjectorSource"])
            else:
                sp.add_new_particles()
        for sp in species:
            sp.free_added()
            sp.sort_parts(grid=grid)
            sp.align_parts()
            nppc = np.int32(np.prod(sp.Args["Nppc"]) + 1)
            sp.Args["right_lim"] = sp.D["x"][-nppc:].max() + 0.5 * sp.Args["ddx"]


# ----------------------------------------------------------------------
def _focus_pulse(EE, w, kx, Xf):
    """laser.py:24-33: spectral E -> (E, G) of the forward-moving pulse
    moved back by Xf."""
    DT = -1.0j * w * np.sign(kx + (kx == 0))
    GG = DT * EE
    EEt = np.cos(w * Xf) * EE + np.sin(w * Xf) / w * GG
    GG = -w * np.sin(w * Xf) * EE + np.cos(w * Xf) * GG
    EE = EEt
    EE *= np.exp(1.0j * kx * Xf)
    GG *= np.exp(1.0j * kx * Xf)
    return EE, GG


def add_gausian_pulse(solver, laser):
    """laser.py:3-37.  Restatement extension without reference code:
    laser["astig"] = a2 (M >= 2) adds the first-order astigmatic term
    Ez_m2 = -(a2/2) (r/R)^2 x the mode-0 profile (the expansion of
    exp(-r^2 (1 + a2 cos 2 phi)/R^2) with fields read as
    F_0 + 2 Re(F_2 e^{-2 i phi})), focused with w_m2."""
    A, D = solver.Args, solver.D
    k0 = 2 * np.pi * laser["k0"]
    a0, Lx, R, x0, xf = (laser[k] for k in ("a0", "Lx", "R", "x0", "x_foc"))
    a2 = float(laser.get("astig", 0.0) or 0.0)
    if a2 and A["M"] < 2:
        raise ValueError("an astigmatic laser (astig != 0) needs M >= 2 modes")
    Xf = x0 - xf
    Xg, Rg = A["Xgrid"], A["Rgrid"]
    kx, w = A["kx"][None, :], A["w_m0"]
    D["Ez_m0"][1:] = (a0 * np.sin(k0 * (Xg[None, :] - x0))
                      * np.exp(-(Xg[None, :] - x0) ** 2 / Lx ** 2 - Rg[1:, None] ** 2 / R ** 2)
                      * (abs(Rg[1:, None]) < 3.5 * R) * (abs(Xg[None, :] - x0) < 3.5 * Lx))
    if a2:
        D["Ez_m2"][1:] = -0.5 * a2 * (Rg[1:, None] / R) ** 2 * D["Ez_m0"][1:]
    solver.fb_transform(scals=["Ez"], dir=0)
    EE, GG = _focus_pulse(D["Ez_fb_m0"].copy(), w, kx, Xf)
    D["Ez_fb_m0"][:] = EE
    D["Gz_fb_m0"][:] = GG
    if a2:
        EE, GG = _focus_pulse(D["Ez_fb_m2"].copy(), A["w_m2"], kx, Xf)
        D["Ez_fb_m2"][:] = EE
        D["Gz_fb_m2"][:] = GG
    solver.restore_B_fb()
    solver.fb_transform(vects=["B", "E"], dir=1)


# ----------------------------------------------------------------------
class OLoop:
    """PIC_loop.step (pic_loop.py:57-142), diagnostics off."""

    def __init__(self, solvers, species, frames=()):
        self.solvers, self.species, self.frames = list(solvers), list(species), list(frames)
        self.main = self.solvers[0]
        self.it = 0

    def step(self):
        for fr in self.frames:
            if np.mod(self.it, fr.Args["Steps"]) == 0:
                fr.shift_grids(grids=self.solvers)
                fr.inject_plasma(species=self.species, grid=self.main)
        for p in self.species:
            p.push_coords("half")
            p.sort_parts(grid=self.main)
        for s in self.solvers:
            s.depose_currents(species=self.species)
        for p in self.species:
            p.push_coords("half")
            p.sort_parts(grid=self.main)
        for s in self.solvers:
            s.depose_charge(species=self.species)
            s.fb_transform(scals=["rho"], vects=["J"], dir=0)
            s.fields_smooth(flds=["rho", "Jx", "Jy", "Jz"])
            for m in range(s.Args["M"] + 1):
                for c in VEC:
                    s.D["dN0" + c + "_fb_m" + str(m)][:] = s.D["dN1" + c + "_fb_m" + str(m)]
            s.field_grad("rho", "dN1")
            s.push_fields()
            s.damp_fields()
            s.restore_B_fb()
            s.fb_transform(vects=["E", "B"], dir=1)
            s.gather_and_push(species=self.species)
        self.it += 1
        return self.it


# ----------------------------------------------------------------------
def diagnostics(solver, species):
    """Integrated diagnostics (defined identically for the oracle and the
    product): field energy  sum_m w_m sum (|E|^2+|B|^2) 2 pi r dr dx  over the
    physical rows r > 0 (w_0 = 1, w_m>=1 = 2); on-axis amplitudes
    max |Ez_m0[1, :]| (the laser's polarisation component: x is the
    propagation axis in these arrays) and max |Ex_m0[1, :]| (the longitudinal
    field on the axis, the plasma wake: a linearly polarised laser has no
    mode-0 longitudinal field); kinetic energy sum w (gamma - 1) of the
    mobile species."""
    A, D = solver.Args, solver.D
    r = A["Rgrid"][1:, None]
    vol = 2 * np.pi * r * A["dr"] * A["dx"]
    We = 0.0
    for m in range(A["M"] + 1):
        wm = 1.0 if m == 0 else 2.0
        for f in ("E", "B"):
            for c in VEC:
                a = D[f + c + "_m" + str(m)][1:]
                We += wm * float((np.abs(a) ** 2 * vol).sum())
    ez = np.abs(D["Ez_m0"][1])
    ex = np.abs(D["Ex_m0"][1])
    kin = 0.0
    for p in species:
        if "Immobile" in p.Args or p.Args["Np"] == 0:
            continue
        kin += float((p.D["w"] * (1.0 / p.D["g_inv"] - 1.0)).sum())
    return {"field_energy": We, "ez_axis_max": float(ez.max()), "wake_ex_max": float(ex.max()),
            "kinetic": kin}


def build_lpa(grid_in, eons_in, frame_in=None, laser_in=None, prefill=None, K=None, seed=0,
              density_profiles=None, ion_mass=None):
    """Set up solver + electrons + immobile ions (+ frame, laser, prefilled
    window) the way the reference's example scripts do
    (examples/lpa_script_small.py:51-95); with ion_mass the ions are a
    second mobile species of that mass."""
    K = K or get_kernels("port")
    solver = OGrid(copy.deepcopy(grid_in), K)
    if laser_in is not None:
        add_gausian_pulse(solver, laser_in)
    e_in = copy.deepcopy(eons_in)
    e_in.update(dx=solver.Args["dx"], dr=solver.Args["dr"], dt=solver.Args["dt"])
    i_in = copy.deepcopy(e_in)
    i_in["charge"] = 1
    if ion_mass is None:
        i_in["Immobile"] = True
    else:
        i_in["mass"] = ion_mass
    eons = OSpecies(e_in, K, seed=seed)
    ions = OSpecies(i_in, K, seed=seed + 1)
    ions.Args["InjectorSource"] = eons
    if prefill is not None:
        dom = dict(prefill)
        eons.make_new_domain(dom, density_profiles=density_profiles)
        eons.add_new_particles()
        ions.add_new_particles(source=eons)
        eons.free_added()
    frames = []
    if frame_in is not None:
        f_in = dict(frame_in)
        f_in["dt"] = solver.Args["dt"]
        f_in.setdefault("DensityProfiles", density_profiles)
        frames.append(OFrame(f_in))
    loop = OLoop([solver], [eons, ions], frames)
    return solver, eons, ions, loop
