"""Maxwell-solver methods (the CUDA counterpart of
chimeraCL/methods/solver_methods_cl.py): PSATD update and absorbing edges."""
import numpy as np

from .._lib import PP, call, stream
from .generic_methods_cu import GenericMethodsCU


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
