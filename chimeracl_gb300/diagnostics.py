"""Field and particle records (the reference's chimeraCL/diagnostics.py).

One record per ``Interval`` iterations, named by the 9-digit zero-padded
iteration, with the reference's path convention (diagnostics.py:1-15):

* ``/data/fields/<name>``: real-space field of every azimuthal mode, stacked
  as [m=0, Re m=1, Im m=1, Re m=2, ...] along axis 0, shape (1 + 2M, Nr, Nx),
  in ``dtype_flds``;
* ``/data/species/species_<i>/<component>``: the listed particle components
  of species i (optionally selected by value ranges), weights scaled by
  ``w2pC`` to pC (the diagnostics' ``w2pC`` if given, else the species'),
  in ``dtype_parts``;
* ``/data/info/``: iteration, Xgrid, Rgrid, dx, dr, dt, Nx, Nr, M,
  FrameVelocity.

The record is an HDF5 file (``<it>.h5``) when h5py can be imported, as in the
reference; otherwise the same paths are the keys of a numpy archive
(``<it>.npz``, one array per path).  ``read_record`` reads either back into a
flat {path: array} dict.

As in the reference (diagnostics.py:126-131), writing ``rho`` or a current
component first re-deposits the charge, then takes the field forward,
smooths it and brings it back: the record of ``rho`` is the charge density
of the species at the recorded iteration after the smoothing filter, and a
record changes the solver's scratch arrays (not the fields that the next
step reads)."""
import os

import numpy as np

try:  # the reference's format, where available
    import h5py
except ImportError:  # neither this image nor its GPU hosts ship h5py
    h5py = None


class _Record:
    """One output file: HDF5 through h5py, else a numpy archive."""

    def __init__(self, base):
        self._h5 = h5py.File(base + ".h5", "w") if h5py is not None else None
        self._base = base
        self._items = {}

    def __setitem__(self, path, value):
        if self._h5 is not None:
            self._h5[path] = value
        else:
            self._items[path.lstrip("/")] = np.asarray(value)

    def close(self):
        if self._h5 is not None:
            self._h5.close()
        else:
            np.savez(self._base + ".npz", **self._items)


def read_record(fname):
    """A record as {"/data/...": ndarray}, from either file format."""
    out = {}
    if fname.endswith(".h5"):
        if h5py is None:
            raise RuntimeError("reading an HDF5 record needs h5py")
        with h5py.File(fname, "r") as f:
            f.visititems(lambda name, obj: out.__setitem__(
                "/" + name, obj[()]) if isinstance(obj, h5py.Dataset) else None)
        return out
    with np.load(fname) as z:
        for k in z.files:
            out["/" + k] = z[k]
    return out


class Diagnostics:
    """diagnostics.py:21-52: ``configs_in`` holds ``Interval`` and optionally
    ``ScalarFields`` (e.g. ['rho', 'Ez']), ``VectorFields`` (e.g. ['E'],
    written per component), ``Species`` ({'Components': [...],
    'Selections': [(component, vmin, vmax), ...]}).  ``path`` is relative to
    the working directory; an existing directory is emptied."""

    def __init__(self, configs_in, solver, species=(), frame=None, path="diags",
                 dtype_flds=np.float32, dtype_parts=np.float64):
        self.Args = configs_in
        self.solver = solver
        self.species = list(species)
        self.frame = frame
        self.dtype_flds = dtype_flds
        self.dtype_parts = dtype_parts
        self.base_str = "/data/"
        self.flds_str = "fields/"
        self.parts_str = "species/"
        self.info_str = "info/"
        self.generic_keys = ["Xgrid", "Rgrid", "dx", "dr", "dt", "Nx", "Nr", "M"]
        self.path = os.path.join(os.getcwd(), path) + "/"
        if not os.path.exists(self.path):
            os.makedirs(self.path)
        else:
            for fl in os.listdir(self.path):
                os.remove(self.path + fl)
        self.Args.setdefault("ScalarFields", [])
        self.Args.setdefault("VectorFields", [])
        self.Args.setdefault("Species", {"Components": []})
        self.record = None

    def make_record(self, it):
        """diagnostics.py:54-75"""
        if np.mod(it, self.Args["Interval"]) != 0:
            return
        self.record = _Record(self.path + str(it).zfill(9))
        self.record[self.base_str + self.info_str + "iteration"] = it
        self.add_generic_info()
        for fld in self.Args["ScalarFields"]:
            self.add_field(fld)
        for fld in self.Args["VectorFields"]:
            for comp in ("x", "y", "z"):
                self.add_field(fld + comp)
        self.add_species()
        self.record.close()
        self.record = None

    def add_species(self):
        """diagnostics.py:77-110"""
        for i, part in enumerate(self.species):
            h5_path = self.base_str + self.parts_str + "species_" + str(i) + "/"
            Np = int(part.Args["Np"])
            indx = None
            if "Selections" in self.Args["Species"] and Np > 0:
                mask = np.ones(Np, dtype=bool)
                for comp_select, vmin, vmax in self.Args["Species"]["Selections"]:
                    v = part.DataDev[comp_select][:Np].cpu().numpy()
                    if vmin is not None:
                        mask &= v > vmin
                    if vmax is not None:
                        mask &= v < vmax
                indx = np.nonzero(mask)
            for comp in self.Args["Species"]["Components"]:
                if Np == 0:
                    vals = np.array([], dtype=self.dtype_parts)
                else:
                    vals = part.DataDev[comp][:Np].cpu().numpy()
                    vals = (vals if indx is None else vals[indx]).astype(self.dtype_parts)
                if comp == "w":
                    # the reference reads w2pC from the diagnostics' own
                    # configs (a KeyError when absent there); the species
                    # carries the same factor (particles.py:96)
                    w2pC = self.Args.get("w2pC", part.Args["w2pC"])
                    vals = vals * self.dtype_parts(w2pC)
                self.record[h5_path + comp] = vals

    def add_generic_info(self):
        """diagnostics.py:112-119"""
        h5_path = self.base_str + self.info_str
        for key in self.generic_keys:
            self.record[h5_path + key] = self.solver.Args[key]
        vel = 0.0 if self.frame is None else self.frame.Args["Velocity"]
        self.record[h5_path + "FrameVelocity"] = vel

    def add_field(self, fld):
        """diagnostics.py:121-141"""
        sol = self.solver
        if fld == "rho" or fld[0] == "J":
            # the deposit reads the cell sort; a record taken before the
            # first step finds none (the reference then fails on the missing
            # cell_offset): sort first -- indices only, no particle moves
            for sp in self.species:
                sp.sort_parts(grid=sol)
            sol.depose_charge(self.species)
            sol.fb_transform(scals=[fld], dir=0)
            sol.fields_smooth(flds=[fld])
        sol.fb_transform(scals=[fld], dir=1)
        stack = [sol.DataDev[fld + "_m0"].cpu().numpy()[None].astype(self.dtype_flds)]
        for m in range(1, sol.Args["M"] + 1):
            f = sol.DataDev[fld + "_m" + str(m)].cpu().numpy()[None]
            stack.append(f.real.astype(self.dtype_flds))
            stack.append(f.imag.astype(self.dtype_flds))
        self.record[self.base_str + self.flds_str + fld] = np.concatenate(stack, axis=0)
