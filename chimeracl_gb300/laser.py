"""Gaussian laser pulse initialisation (the reference's chimeraCL/laser.py).

The pulse envelope is written into Ez of mode 0 on the host, transformed,
focused analytically in spectral space, and E, G, B are restored from it."""
import numpy as np
import torch


def add_gausian_pulse(solver, laser):
    """laser.py:3-37; laser = {k0, a0, x0, Lx, R, x_foc}."""
    k0 = 2 * np.pi * laser["k0"]
    a0, Lx, R = laser["a0"], laser["Lx"], laser["R"]
    x0, x_foc = laser["x0"], laser["x_foc"]
    X_focus = x0 - x_foc
    Xg, Rg = solver.Args["Xgrid"], solver.Args["Rgrid"]
    kx, w = solver.Args["kx"][None, :], solver.Args["w_m0"]
    D = solver.DataDev
    ez = (a0 * np.sin(k0 * (Xg[None, :] - x0))
          * np.exp(-(Xg[None, :] - x0) ** 2 / Lx ** 2 - Rg[1:, None] ** 2 / R ** 2)
          * (abs(Rg[1:, None]) < 3.5 * R) * (abs(Xg[None, :] - x0) < 3.5 * Lx))
    D["Ez_m0"][1:] = torch.from_numpy(ez).to(D["Ez_m0"].dtype)
    solver.fb_transform(scals=["Ez"], dir=0)
    EE = D["Ez_fb_m0"].cpu().numpy().astype(np.complex128)
    DT = -1.0j * w * np.sign(kx + (kx == 0))
    GG = DT * EE
    EE_t = np.cos(w * X_focus) * EE + np.sin(w * X_focus) / w * GG
    GG = -w * np.sin(w * X_focus) * EE + np.cos(w * X_focus) * GG
    EE = EE_t
    EE *= np.exp(1.0j * kx * X_focus)
    GG *= np.exp(1.0j * kx * X_focus)
    D["Ez_fb_m0"].copy_(torch.from_numpy(EE).to(D["Ez_fb_m0"].dtype))
    D["Gz_fb_m0"].copy_(torch.from_numpy(GG).to(D["Gz_fb_m0"].dtype))
    solver.restore_B_fb()
    solver.fb_transform(vects=["B", "E"], dir=1)
