"""Grid wrapper (the reference's chimeraCL/grid.py): geometry, real-space
mode fields, deposit and gather entry points."""
import numpy as np

from .methods.generic_methods_cu import ArgsDict
from .methods.grid_methods_cu import GridMethodsCU


class Grid(GridMethodsCU):
    def __init__(self, configs_in, comm):
        self.import_comm(comm)
        self.set_global_working_group_size()
        self._process_configs(configs_in)
        if "vec_comps" not in self.Args:
            self.Args["vec_comps"] = ["x", "y", "z"]
        self.init_grid_methods()
        self.DataDev = {}
        self._init_grid_data_on_dev()
        self.send_args_to_dev()

    def depose_charge(self, species=(), zero=True):
        """rho = sum over species of the charge deposit, then axis and 1/dV
        (grid.py:23-31).  zero=False: rho was cleared already (the loop
        clears it with J, in one launch)."""
        if zero:
            self.set_many([self.DataDev["rho_m" + str(m)] for m in range(self.Args["M"] + 1)], 0)
        for parts in species:
            self.depose_scalar(parts, "w", "rho", charge=parts.Args["charge"])
        self.postproc_depose_scalar("rho")

    def depose_currents(self, species=(), also_zero=()):
        """J from the mobile species (grid.py:33-54).  also_zero: scalar
        fields (e.g. "rho") cleared in the same launch as J."""
        M = self.Args["M"]
        self.set_many([self.DataDev["J" + c + "_m" + str(m)]
                       for m in range(M + 1) for c in self.Args["vec_comps"]]
                      + [self.DataDev[f + "_m" + str(m)] for f in also_zero for m in range(M + 1)],
                      0)
        mom = ["p" + c for c in self.Args["vec_comps"]]
        for parts in species:
            if "Immobile" in parts.Args:
                continue
            self.depose_vector(parts, mom, ["g_inv", "w"], "J", charge=parts.Args["charge"])
        self.postproc_depose_vector("J")

    def gather_and_push(self, species=()):
        """Ghost rows of E, B, then gather + Boris push of the mobile species
        (grid.py:56-66)."""
        self.preproc_project_vecs(("E", "B"))  # both fields' ghost rows, one launch
        for parts in species:
            if "Immobile" in parts.Args:
                continue
            self._gather_and_push(parts, ["E", "B"])

    def _process_configs(self, configs_in):
        """Grid geometry, as grid.py:68-103: dx over Nx-1 intervals, radial
        nodes at (ir - 1/2) dr, 1/dV with the ghost row r < 0 masked."""
        A = self.Args = configs_in if isinstance(configs_in, ArgsDict) else ArgsDict(configs_in)
        if "M" not in A:
            A["M"] = 0
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
        A["dont_send"] = []
        A["dont_keep"] = []

    def _init_grid_data_on_dev(self):
        """E, B, J, G (3 components) and rho per mode: m=0 real (Nr, Nx),
        m>=1 complex (grid.py:106-127)."""
        names = [f + c for f in ("E", "B", "J", "G") for c in self.Args["vec_comps"]] + ["rho"]
        shape = (self.Args["Nr"], self.Args["Nx"])
        for n in names:
            self.DataDev[n + "_m0"] = self.dev_arr(val=0, shape=shape, dtype=self.comm.real)
            for m in range(1, self.Args["M"] + 1):
                self.DataDev[n + "_m" + str(m)] = self.dev_arr(val=0, shape=shape,
                                                               dtype=self.comm.cplx)
