"""Grid methods (the CUDA counterpart of chimeraCL/methods/grid_methods_cl.py):
charge/current deposit, deposit post-processing, ghost-row fill and the
field gather + Boris push."""
import numpy as np

from .._lib import PP, call, stream
from .generic_methods_cu import GenericMethodsCU


class GridMethodsCU(GenericMethodsCU):
    def init_grid_methods(self):
        self.init_generic_methods()
        if not 0 <= self.Args["M"] <= 3:
            raise ValueError("chimeracl_gb300 handles azimuthal modes M = 0..3")
        if "vec_comps" not in self.Args:
            self.Args["vec_comps"] = ["x", "y", "z"]

    def _grid_scalars(self):
        A = self.Args
        return (A["Nx"], float(A["Xmin"]), float(A["dx_inv"]), A["Nr"], float(A["Rmin"]),
                float(A["dr_inv"]))

    def _real_dev(self, name):
        """Device copy of a real coefficient array in the compute precision."""
        t = self.DataDev[name]
        if t.dtype == self.comm.real:
            return t
        key = "_" + name + "_" + str(self.comm.real).split(".")[-1]
        if key not in self.DataDev or self.DataDev[key].shape != t.shape:
            self.DataDev[key] = t.to(self.comm.real).contiguous()
        return self.DataDev[key]

    def depose_scalar(self, parts, src_scalar, dest_fld, charge):
        """grid_methods_cl.py:44-69 (one launch instead of four colours)."""
        if parts.Args["Np"] <= 0:
            return
        D, M = parts.DataDev, self.Args["M"]
        flds = [self.DataDev[dest_fld + "_m" + str(m)] for m in range(M + 1)]
        args = [self._dt, M, D["sort_indx"].data_ptr(), D["cell_offset"].data_ptr(),
                D["x"].data_ptr(), D["y"].data_ptr(), D["z"].data_ptr(),
                D[src_scalar].data_ptr(), int(np.int8(charge)), *self._grid_scalars(), PP(flds)]
        if "x_lo" in D:  # compensated coordinates: fractions from hi + lo
            call("ccl_deposit_scalar_lo", *args, *self._low_parts(D), stream())
        else:
            call("ccl_deposit_scalar", *args, stream())

    @staticmethod
    def _low_parts(D):
        return [D[k].data_ptr() for k in ("x_lo", "y_lo", "z_lo")]

    def depose_vector(self, parts, vec, factors, vec_fld, charge):
        """grid_methods_cl.py:71-95; factors = [g_inv, w]."""
        if parts.Args["Np"] <= 0:
            return
        D, M = parts.DataDev, self.Args["M"]
        flds = [self.DataDev[vec_fld + c + "_m" + str(m)]
                for m in range(M + 1) for c in self.Args["vec_comps"]]
        args = [self._dt, M, D["sort_indx"].data_ptr(), D["cell_offset"].data_ptr(),
                D["x"].data_ptr(), D["y"].data_ptr(), D["z"].data_ptr(), D[vec[0]].data_ptr(),
                D[vec[1]].data_ptr(), D[vec[2]].data_ptr(), D[factors[0]].data_ptr(),
                D[factors[1]].data_ptr(), int(np.int8(charge)), *self._grid_scalars(), PP(flds)]
        if "x_lo" in D:
            call("ccl_deposit_vector_lo", *args, *self._low_parts(D), stream())
        else:
            call("ccl_deposit_vector", *args, stream())

    def _postproc(self, names):
        M = self.Args["M"]
        flds = [self.DataDev[f + "_m" + str(m)] for f in names for m in range(M + 1)]
        call("ccl_deposit_postproc", self._dt, M, len(names), PP(flds), self.Args["Nx"],
             self.Args["Nr"], self._real_dev("dV_inv").data_ptr(), stream())

    def postproc_depose_scalar(self, fld):
        """grid_methods_cl.py:98-124"""
        self._postproc([fld])

    def postproc_depose_vector(self, vec_fld):
        """grid_methods_cl.py:126-151"""
        self._postproc([vec_fld + c for c in self.Args["vec_comps"]])

    def preproc_project_vec(self, vec_fld):
        """grid_methods_cl.py:153-166"""
        self.preproc_project_vecs((vec_fld,))

    def preproc_project_vecs(self, vec_flds):
        """preproc_project_vec of several vector fields in one launch."""
        M = self.Args["M"]
        names = [v + c for v in vec_flds for c in self.Args["vec_comps"]]
        flds = [self.DataDev[f + "_m" + str(m)] for f in names for m in range(M + 1)]
        call("ccl_warp_axis", self._dt, M, len(names), PP(flds), self.Args["Nx"], stream())

    def _gather_and_push(self, parts, flds):
        """grid_methods_cl.py:168-192"""
        if parts.Args["Np"] == 0:
            return
        D, M = parts.DataDev, self.Args["M"]
        f = [self.DataDev[fl + c + "_m" + str(m)]
             for m in range(M + 1) for fl in flds for c in self.Args["vec_comps"]]
        # with the sort's cell offsets (the FP32 form runs tile by tile)
        args = [self._dt, M, parts.Args["Np"], D["x"].data_ptr(), D["y"].data_ptr(),
                D["z"].data_ptr(), D["px"].data_ptr(), D["py"].data_ptr(), D["pz"].data_ptr(),
                D["g_inv"].data_ptr(), D["sort_indx"].data_ptr(), D["cell_offset"].data_ptr(),
                D["Np_stay_dev"].data_ptr(), float(parts.Args["FactorPush"]),
                *self._grid_scalars(), PP(f)]
        if "x_lo" in D:
            call("ccl_gather_push_cells_lo", *args, *self._low_parts(D), stream())
        else:
            call("ccl_gather_push_cells", *args, stream())
