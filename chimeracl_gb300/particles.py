"""Particles wrapper (the reference's chimeraCL/particles.py): species
configuration and its structure-of-arrays device data."""
import numpy as np
import torch

from .methods.generic_methods_cu import ArgsDict
from .methods.particles_methods_cu import ParticleMethodsCU

# SI constants used for the weight-to-charge factor w2pC (particles.py:96)
_M_E, _C, _E, _EPS0 = 9.1093837015e-31, 299792458.0, 1.602176634e-19, 8.8541878128e-12


class Particles(ParticleMethodsCU):
    def __init__(self, configs_in, comm=None, seed=None):
        self.import_comm(comm)
        self.set_global_working_group_size()
        self.DataDev = {}
        self._seed = seed
        self.init_particle_methods()
        self._process_configs(configs_in)
        self.send_args_to_dev()
        self._init_data_on_dev()

    def sort_parts(self, grid):
        """Cell sort unless already sorted (particles.py:23-29)."""
        if self.Args["Np"] == 0:
            self.flag_sorted = True
        if not self.flag_sorted:
            self.index_sort(grid)
            self.flag_sorted = True

    def add_particles(self, domain_in=None, beam_in=None, source=None):
        """particles.py:31-41"""
        if source is None:
            if domain_in is not None:
                self.make_new_domain(domain_in)
            elif beam_in is not None:
                self.make_new_beam(beam_in)
            self.add_new_particles()
        else:
            self.add_new_particles(source=source)

    def align_parts(self):
        """Permute into cell order and drop leavers (particles.py:43-51)."""
        if self.Args["Np"] == 0:
            return
        self.align_and_damp(comps_align=self._comps())

    def align_begin(self):
        """align_parts in two halves, for several species at a window shift:
        this one queues the permutation and reads nothing back ..."""
        self._align_state = None
        if self.Args["Np"] != 0:
            self._align_state = self.align_queue(self._comps())

    def align_end(self):
        """... this one reads the in-window count and cuts the arrays to it."""
        state, self._align_state = getattr(self, "_align_state", None), None
        if state is not None:
            self.align_finish(state)

    def _process_configs(self, configs_in):
        """particles.py:53-100"""
        A = self.Args = configs_in if isinstance(configs_in, ArgsDict) else ArgsDict(configs_in)
        A["Np"] = 0
        A["Np_stay"] = 0
        for k, v in (("dt", 1.0), ("dx", 1.0), ("dr", 1.0), ("charge", -1.0), ("mass", 1.0),
                     ("dens", 1.0)):
            if k not in A:
                A[k] = v
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
        A["w2pC"] = 4 * np.pi ** 2 * _M_E * _C ** 2 * _EPS0 * 1e6 / _E
        A["dont_send"] = ["InjectorSource", "charge", "mass", "dens", "Immobile", "w2pC"]
        A["dont_keep"] = []

    def _init_data_on_dev(self):
        for arg in self._comps():
            self.DataDev[arg] = torch.zeros(0, dtype=self.comm.real, device=self.comm.device)
        self.DataDev["Np_stay_dev"] = torch.zeros(1, dtype=torch.int32, device=self.comm.device)
        if "Np" not in self.DataDev:
            self.DataDev["Np"] = torch.zeros(1, dtype=torch.int64, device=self.comm.device)
