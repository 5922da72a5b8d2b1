"""Solver wrapper (the reference's chimeraCL/solver.py): grid + transformer
+ PSATD coefficients; push, damp and B-restore entry points."""
import numpy as np
import torch

from ._lib import PP, call, ints, stream
from .grid import Grid
from .methods.solver_methods_cu import SolverMethodsCU, psatd_split_coefficients
from .transformer import Transformer


class Solver(Grid, Transformer, SolverMethodsCU):
    def __init__(self, configs_in, comm):
        self.import_comm(comm)
        self.set_global_working_group_size()
        self._process_configs(configs_in)
        self.Args["vec_comps"] = ["x", "y", "z"]
        self.init_solver_methods()
        self.init_grid_methods()
        self.DataDev = {}
        self._init_grid_data_on_dev()
        self.init_transformer()
        self._make_ms_coefficients()
        self.send_args_to_dev()

    def push_fields(self):
        """PSATD advance of E, G (solver.py:29-30)."""
        self.advance_fields(vecs=["E", "G", "J", "dN0", "dN1"])

    def damp_fields(self):
        """Absorbing edges in (x, kr) space (solver.py:32-35): half backward
        transform, edge profile, half forward transform -- one fused kernel
        per field component and mode."""
        A = self.Args
        nf = 2 * int(self._damp_cells())
        pp, pm = self._phase(1), self._phase(0)
        prof = self._real_dev("DampProfile")
        ent = [(f + c, m) for f in ("E", "G") for c in A["vec_comps"] for m in range(A["M"] + 1)]
        for k in range(0, len(ent), 32):
            part = ent[k:k + 32]
            sp = [self.DataDev[n + "_fb_m" + str(m)] for n, m in part]
            rs = [self.DataDev[n + "_m" + str(m)] for n, m in part]
            call("ccl_damp_batch", self._dt, len(part), A["Nr"] - 1, A["Nx"], PP(sp), PP(rs),
                 ints([int(m == 0) for _, m in part]), pp.data_ptr(), pm.data_ptr(),
                 prof.data_ptr(), nf, stream())

    def restore_B_fb(self):
        """B = rot(G) / w^2 in spectral space (solver.py:37-39); the 1/w^2
        factor (field_poiss_vec) is applied in the curl's combine pass."""
        self.field_rot("G", "B", poisson=True)

    def _make_ms_coefficients(self):
        """cos(w dt), sin(w dt) w and 1/w^2 per mode (solver.py:41-52), in
        float64 on the host; with FP32 fields also the eight coefficients of
        the cancellation-free form of the update."""
        for m in range(self.Args["M"] + 1):
            w = self.Args["w_m" + str(m)]
            dt = self.Args["dt"]
            self.Args["MxSlv_cos(wdt)_m" + str(m)] = np.cos(w * dt)
            self.Args["MxSlv_sin(wdt)*w_m" + str(m)] = np.sin(w * dt) * w
            self.Args["MxSlv_1/w**2_m" + str(m)] = 1.0 / w ** 2
            for k in ("MxSlv_cos(wdt)_m", "MxSlv_sin(wdt)*w_m", "MxSlv_1/w**2_m"):
                self.Args["dont_keep"].append(k + str(m))
            comm = getattr(self, "comm", None)
            if comm is not None and comm.real != torch.float64:
                # FP32 fields: the cancellation-free form of the same update
                self.Args["MxSlv_split_m" + str(m)] = psatd_split_coefficients(w, dt).astype(
                    np.float32)
                self.Args["dont_keep"].append("MxSlv_split_m" + str(m))
