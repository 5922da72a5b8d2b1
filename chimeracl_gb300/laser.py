"""Gaussian laser pulse initialisation (the reference's chimeraCL/laser.py).

The pulse envelope is written into Ez of mode 0 on the host, transformed,
focused analytically in spectral space, and E, G, B are restored from it.

Optional astigmatism (``laser["astig"] = a2``, no counterpart in the
reference; needs M >= 2): the transverse profile exp(-y^2/Ry^2 - z^2/Rz^2)
with 1/Ry^2 = (1 + a2)/R^2 and 1/Rz^2 = (1 - a2)/R^2 is taken to first order
in a2, exp(-r^2/R^2) (1 - a2 (r/R)^2 cos 2 phi), where r^2 cos 2 phi = y^2 - z^2
and e^{i phi} = (y + i z)/r as in the deposits.  With fields read as
F_0 + 2 Re(F_2 e^{-2 i phi}) that is an m = 2 term
Ez_m2 = -(a2/2) (r/R)^2 times the mode-0 profile (regular on the axis, as
r^2), focused like mode 0 with mode 2's dispersion w_m2."""
import numpy as np
import torch


def _focus(EE, w, kx, X_focus):
    """Spectral E of a pulse -> (E, G) of the forward-moving pulse moved
    back by X_focus (laser.py:24-33), in float64."""
    DT = -1.0j * w * np.sign(kx + (kx == 0))
    GG = DT * EE
    EE_t = np.cos(w * X_focus) * EE + np.sin(w * X_focus) / w * GG
    GG = -w * np.sin(w * X_focus) * EE + np.cos(w * X_focus) * GG
    EE = EE_t
    EE *= np.exp(1.0j * kx * X_focus)
    GG *= np.exp(1.0j * kx * X_focus)
    return EE, GG


def add_gausian_pulse(solver, laser):
    """laser.py:3-37; laser = {k0, a0, x0, Lx, R, x_foc} and optionally
    astig (the m = 2 astigmatic fraction a2, module docstring)."""
    k0 = 2 * np.pi * laser["k0"]
    a0, Lx, R = laser["a0"], laser["Lx"], laser["R"]
    x0, x_foc = laser["x0"], laser["x_foc"]
    X_focus = x0 - x_foc
    Xg, Rg = solver.Args["Xgrid"], solver.Args["Rgrid"]
    kx, w = solver.Args["kx"][None, :], solver.Args["w_m0"]
    D = solver.DataDev
    a2 = float(laser.get("astig", 0.0) or 0.0)
    if a2 and solver.Args["M"] < 2:
        raise ValueError("an astigmatic laser (astig != 0) needs M >= 2 modes")
    ez = (a0 * np.sin(k0 * (Xg[None, :] - x0))
          * np.exp(-(Xg[None, :] - x0) ** 2 / Lx ** 2 - Rg[1:, None] ** 2 / R ** 2)
          * (abs(Rg[1:, None]) < 3.5 * R) * (abs(Xg[None, :] - x0) < 3.5 * Lx))
    D["Ez_m0"][1:] = torch.from_numpy(ez).to(D["Ez_m0"].dtype)
    if a2:
        ez2 = -0.5 * a2 * (Rg[1:, None] / R) ** 2 * ez
        D["Ez_m2"][1:] = torch.from_numpy(ez2).to(D["Ez_m2"].dtype)
    solver.fb_transform(scals=["Ez"], dir=0)
    EE = D["Ez_fb_m0"].cpu().numpy().astype(np.complex128)
    EE, GG = _focus(EE, w, kx, X_focus)
    D["Ez_fb_m0"].copy_(torch.from_numpy(EE).to(D["Ez_fb_m0"].dtype))
    D["Gz_fb_m0"].copy_(torch.from_numpy(GG).to(D["Gz_fb_m0"].dtype))
    if a2:
        EE2 = D["Ez_fb_m2"].cpu().numpy().astype(np.complex128)
        EE2, GG2 = _focus(EE2, solver.Args["w_m2"], kx, X_focus)
        D["Ez_fb_m2"].copy_(torch.from_numpy(EE2).to(D["Ez_fb_m2"].dtype))
        D["Gz_fb_m2"].copy_(torch.from_numpy(GG2).to(D["Gz_fb_m2"].dtype))
    solver.restore_B_fb()
    solver.fb_transform(vects=["B", "E"], dir=1)
