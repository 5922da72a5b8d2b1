"""Maxwell-solver methods (the CUDA counterpart of
chimeraCL/methods/solver_methods_cl.py): PSATD update and absorbing edges."""
import numpy as np

from .._lib import PP, call, stream
from .generic_methods_cu import GenericMethodsCU


def psatd_split_coefficients(w, dt):
    """The eight per-cell coefficients of ccl_psatd_advance_split, in
    float64, shape w.shape + (8,): cos x, w sin x, s = sin x / w, 2 pi s,
    2 pi (1 - cos x), 2 pi (cos x - sin x / x) / w^2,
    2 pi (sin x / x - 1) / w^2, 2 pi (1 - cos x) / (w^2 dt), x = w dt.
    The two differences of O(1) terms go by their Taylor series below
    x = 0.1 (to x^10: truncation below 1e-19 relative), 1 - cos x as
    2 sin^2(x/2)."""
    w = np.asarray(w, dtype=np.float64)
    x = w * dt
    sx, cx = np.sin(x), np.cos(x)
    one_m_cos = 2.0 * np.sin(0.5 * x) ** 2
    x2 = x * x
    small = x < 0.1
    xs = np.where(small, 1.0, x)  # the direct forms only where x >= 0.1
    # (cos x - sin x / x) / w^2 and (sin x / x - 1) / w^2
    a_ser = dt * dt * (-1.0 / 3 + x2 * (1.0 / 30 + x2 * (-1.0 / 840 + x2 * (
        1.0 / 45360 - x2 / 3991680))))
    b_ser = dt * dt * (-1.0 / 6 + x2 * (1.0 / 120 + x2 * (-1.0 / 5040 + x2 * (
        1.0 / 362880 - x2 / 39916800))))
    a_dir = (cx - sx / xs) / w ** 2
    b_dir = (sx / xs - 1.0) / w ** 2
    a = np.where(small, a_ser, a_dir)
    b = np.where(small, b_ser, b_dir)
    s = sx / w
    pi2 = 2.0 * np.pi
    return np.stack([cx, w * sx, s, pi2 * s, pi2 * one_m_cos, pi2 * a, pi2 * b,
                     pi2 * one_m_cos / (w ** 2 * dt)], axis=-1)


class SolverMethodsCU(GenericMethodsCU):
    def init_solver_methods(self):
        if "DampCells" in self.Args:
            self._init_field_damping()

    def _init_field_damping(self):
        """sin^2 absorbing profile over 2*DampCells cells
        (solver_methods_cl.py:32-41)."""
        N = int(self.Args["DampCells"])
        z = np.arange(2 * N)
        z_shft = 3.0 * (z - N + 1) / (N + 1)
        prof = (z < 4.0 * N / 3) * (z >= N) * np.sin(0.5 * np.pi * z_shft) ** 2 + (z >= 4.0 * N / 3)
        self.Args["DampProfile"] = prof.astype(np.float64)
        self.Args["dont_keep"].append("DampProfile")
        self.Args["dont_send"].append("DampCells")

    def advance_fields(self, vecs):
        """PSATD update of E, G per mode (solver_methods_cl.py:43-62)."""
        A = self.Args
        n = A["NxNrm1"]
        for m in range(A["M"] + 1):
            s = "_m" + str(m)
            flds = [self.DataDev[v + c + "_fb" + s] for v in vecs for c in A["vec_comps"]]
            if "MxSlv_split" + s in self.DataDev:  # FP32 fields
                call("ccl_psatd_advance_split", self._dt, n,
                     self.DataDev["MxSlv_split" + s].data_ptr(), PP(flds), stream())
                continue
            call("ccl_psatd_advance", self._dt, n, float(A["dt_inv"]),
                 self._real_dev("MxSlv_cos(wdt)" + s).data_ptr(),
                 self._real_dev("MxSlv_sin(wdt)*w" + s).data_ptr(),
                 self._real_dev("MxSlv_1/w**2" + s).data_ptr(), PP(flds), stream())

    def profile_edges(self, flds):
        """Edge profile on real-space fields (solver_methods_cl.py:64-83)."""
        A = self.Args
        prof = self._real_dev("DampProfile")
        for fld in flds:
            for c in A["vec_comps"]:
                for m in range(A["M"] + 1):
                    a = self.DataDev[fld + c + "_m" + str(m)]
                    call("ccl_profile_edges", self._dt, int(a.is_complex()), A["Nr"], A["Nx"],
                         a.data_ptr(), prof.data_ptr(), 2 * int(self._damp_cells()), stream())

    def _damp_cells(self):
        return self.Args.get("DampCells", self.DataDev["DampProfile"].numel() // 2)
