"""Fourier-Bessel transformer (the reference's chimeraCL/transformer.py):
spectral axes, Hankel and derivative matrices, spectral buffers."""
import numpy as np
from scipy.special import jn, jn_zeros

from .methods.transformer_methods_cu import TransformerMethodsCU


class Transformer(TransformerMethodsCU):
    def init_transformer(self):
        self._init_transformer_data_on_dev()
        self.init_transformer_methods()
        self._make_spectral_axes()
        self._make_DHT()

    def fb_transform(self, scals=(), vects=(), dir=0, mode="full", filt=None):
        """Transform scalar fields and the components of vector fields
        (transformer.py:17-26); ``filt`` fuses a spectral filter per mode
        into the forward transform."""
        names = list(scals) + [v + c for v in vects for c in self.Args["vec_comps"]]
        self.transform_fields(names, dir=dir, mode=mode, filt=filt)

    def _make_spectral_axes(self):
        """kx (numpy fftfreq order), kr_m = j_{m,n}/R, w = |k|, 1/w^2 and the
        sin^2 smoothing filter (transformer.py:28-63)."""
        A = self.Args
        dx, Nx, dr, Nr = A["dx"], A["Nx"], A["dr"], A["Nr"]
        kx = 2 * np.pi * np.fft.fftfreq(Nx, dx)
        R_period = A["Rgrid"][-1] + 0.5 * dr
        A["kx"] = kx
        for m in range(A["M"] + 2):
            A["kr_m" + str(m)] = jn_zeros(m, Nr - 1) / R_period
        for m in range(A["M"] + 1):
            kr = A["kr_m" + str(m)]
            A["w_m" + str(m)] = np.sqrt(kx[None, :] ** 2 + kr[:, None] ** 2)
            A["Poiss_m" + str(m)] = 1.0 / A["w_m" + str(m)] ** 2
            A["SmoothingFilter_m" + str(m)] = (
                (1 - np.sin(0.5 * np.pi * kx[None, :] / kx.max()) ** 2)
                * (1 - np.sin(0.5 * np.pi * kr[:, None] / kr.max()) ** 2))
        for m in range(A["M"] + 2):
            A["dont_send"].append("kr_m" + str(m))
            A["dont_send"].append("w_m" + str(m))
            A["dont_keep"].append("Poiss_m" + str(m))
            A["dont_keep"].append("SmoothingFilter_m" + str(m))

    def _make_DHT(self):
        """Backward Hankel matrix J_m(r kr), forward = its pseudo-inverse, and
        the derivative matrices coupling mode m to m+-1 (transformer.py:65-97).
        Built on the host in float64."""
        A = self.Args
        Rg = A["Rgrid"][1:, None]
        Rp = Rg[-1] + 0.5 * A["dr"]
        for m in range(A["M"] + 1):
            kr0 = jn_zeros(m, A["Nr"] - 1) / Rp
            krp = jn_zeros(m + 1, A["Nr"] - 1) / Rp
            krm = jn_zeros(m - 1, A["Nr"] - 1) / Rp
            A["DHT_inv_m" + str(m)] = jn(m, Rg * kr0)
            A["DHT_m" + str(m)] = np.linalg.pinv(A["DHT_inv_m" + str(m)])
            A["dDHT_plus_m" + str(m)] = A["DHT_m" + str(m)].dot(0.5 * krp * jn(m, Rg * krp))
            A["dDHT_minus_m" + str(m)] = A["DHT_m" + str(m)].dot(0.5 * krm * jn(m, Rg * krm))
            for k in ("DHT_inv_m", "DHT_m", "dDHT_plus_m", "dDHT_minus_m"):
                A["dont_keep"].append(k + str(m))

    def _init_transformer_data_on_dev(self):
        """Spectral fields (complex (Nr-1, Nx)) of rho, E, B, G, J, dN0, dN1,
        the m=-1 buffers and two work buffers of each kind
        (transformer.py:100-132)."""
        A = self.Args
        shape = (A["Nr"] - 1, A["Nx"])
        names = ["rho"] + [f + c for f in ("E", "B", "G", "J", "dN0", "dN1")
                           for c in A["vec_comps"]]
        for n in names:
            for m in range(A["M"] + 1):
                self.DataDev[n + "_fb_m" + str(m)] = self.dev_arr(val=0, shape=shape,
                                                                  dtype=self.comm.cplx)
        for c in A["vec_comps"]:
            self.DataDev["buff_fb_m-1_" + c] = self.dev_arr(val=0, shape=shape,
                                                            dtype=self.comm.cplx)
        self.DataDev["phs_shft"] = self.dev_arr(val=0, shape=A["Nx"], dtype=self.comm.cplx)
        for i in range(2):
            self.DataDev["fld_buff%d_d" % i] = self.dev_arr(val=0, shape=shape, dtype=self.comm.real)
            self.DataDev["fld_buff%d_c" % i] = self.dev_arr(val=0, shape=shape, dtype=self.comm.cplx)
