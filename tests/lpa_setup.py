"""Shared set-up of laser-wakefield (LPA) test cases for the product and the
oracle: same grid, laser, prefilled plasma window, immobile ions, moving
window and seeded injector draws on both sides (the way the reference's
examples/lpa_script_small.py builds its run)."""
import copy

import numpy as np


def small_lpa(Nx=64, Nr=16, M=1, Xmin=-40.0, Xmax=0.0, Rmax=20.0, nppc=(2, 2, 4), dens=1e-3,
              a0=2.0, R=6.0, Lx=3.0, x0=-10.0, x_foc=None, damp=None, steps=20, seed=3,
              profiles=None, prefill=True):
    grid_in = dict(Xmin=Xmin, Xmax=Xmax, Nx=Nx, Rmin=0.0, Rmax=Rmax, Nr=Nr, M=M,
                   DampCells=damp if damp is not None else max(2, min(50, Nx // 8)))
    return dict(
        grid_in=grid_in,
        eons_in=dict(Nppc=tuple(nppc), dens=dens, charge=-1),
        frame_in=dict(Velocity=1.0, Steps=steps),
        laser_in=dict(k0=1.0, a0=a0, x0=x0, Lx=Lx, R=R, x_foc=x0 if x_foc is None else x_foc),
        prefill=dict(Xmin=Xmin, Xmax=Xmax, Rmin=0.0, Rmax=Rmax) if prefill else None,
        profiles=profiles, seed=seed)


def build_product(cfg, precision="fp64", ion_mass=None, **comm_kw):
    """ion_mass: the ions move, with that mass (else they are immobile)."""
    from chimeracl_gb300 import Communicator
    from chimeracl_gb300.frame import Frame
    from chimeracl_gb300.laser import add_gausian_pulse
    from chimeracl_gb300.particles import Particles
    from chimeracl_gb300.pic_loop import PIC_loop
    from chimeracl_gb300.solver import Solver

    seed = cfg["seed"]
    comm = Communicator(precision=precision, seed=seed, **comm_kw)
    solver = Solver(copy.deepcopy(cfg["grid_in"]), comm)
    if cfg["laser_in"] is not None:
        add_gausian_pulse(solver, dict(cfg["laser_in"]))
    e_in = copy.deepcopy(cfg["eons_in"])
    e_in.update(dx=solver.Args["dx"], dr=solver.Args["dr"], dt=solver.Args["dt"])
    i_in = copy.deepcopy(e_in)
    i_in["charge"] = 1
    if ion_mass is None:
        i_in["Immobile"] = True
    else:
        i_in["mass"] = ion_mass
    eons = Particles(e_in, comm, seed=seed)
    ions = Particles(i_in, comm, seed=seed + 1)
    ions.Args["InjectorSource"] = eons
    if cfg["prefill"] is not None:
        eons.make_new_domain(dict(cfg["prefill"]), density_profiles=cfg["profiles"])
        eons.add_new_particles()
        ions.add_new_particles(source=eons)
        eons.free_added()
    frames = []
    if cfg["frame_in"] is not None:
        f_in = dict(cfg["frame_in"])
        f_in["dt"] = solver.Args["dt"]
        f_in["DensityProfiles"] = cfg["profiles"]
        frames.append(Frame(f_in))
    loop = PIC_loop([solver], [eons, ions], frames)
    return solver, eons, ions, loop


def build_oracle(cfg, kind="port", ion_mass=None):
    from oracle import pic_oracle as po
    from oracle.kernels import get_kernels

    K = get_kernels(kind)
    return po.build_lpa(cfg["grid_in"], cfg["eons_in"], cfg["frame_in"], cfg["laser_in"],
                        prefill=cfg["prefill"], K=K, seed=cfg["seed"],
                        density_profiles=cfg["profiles"], ion_mass=ion_mass)


def to_np(t):
    a = t.detach().cpu().numpy()
    return a


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = np.abs(b).max() if b.size else 0.0
    d = np.abs(a.astype(np.complex128) - b.astype(np.complex128)).max() if b.size else 0.0
    if scale == 0.0:
        return 0.0 if d == 0.0 else np.inf
    return float(d / scale)


def field_floor(osolver, key, dens):
    """Physical magnitude a field array is measured against.

    Several arrays of a quasi-neutral plasma are pure rounding residue at
    some steps -- rho_m0 while the ions still sit on the electrons, and the
    fields it drives -- so a ratio to their own maximum compares noise with
    noise.  They are measured against the scale of the quantity instead:
    E, B, G against the largest E/B/G value of the same (real or spectral)
    kind; rho, J against the plasma density (|rho_e| = dens in units of n_c);
    their spectral images against dens times the transform's gain
    (Nx * max row sum of the forward Hankel matrices); the gradients dN
    against that times the largest wavenumber.  The m=-1 buffers hold G's
    mirror at the end of a step."""
    A, D = osolver.Args, osolver.D
    spectral = "_fb" in key
    base = key.split("_")[0]
    if (base[0] in "EBG") or base == "buff":
        grp = [k for k in D if (k[0] in "EBG") and (("_fb" in k) == spectral)]
        return max(float(np.abs(D[k]).max()) for k in grp)
    s = dens
    if spectral:
        M = A["M"]
        s *= A["Nx"] * max(float(np.abs(A["DHT_m%d" % m]).sum(1).max()) for m in range(M + 1))
        if base.startswith("dN"):
            kmax = max([float(np.abs(A["kx"]).max())] +
                       [float(A["kr_m%d" % m].max()) for m in range(M + 2)])
            s *= kmax
    return s


def compare_fields(solver, osolver, keys=None, verbose=False, dens=None):
    """Worst error over the oracle's field arrays: max |a-b| divided by the
    larger of max |b| and the array's physical floor (``field_floor``, used
    when ``dens`` is given; otherwise each array is measured against its own
    maximum)."""
    worst = 0.0
    for k in (keys or osolver.D.keys()):
        # the m=-1 mirror buffers are scratch: the product reads the mirror
        # inside the gradient/curl kernels and no longer materialises them
        if k not in solver.DataDev or k.startswith("buff_fb"):
            continue
        a, b = to_np(solver.DataDev[k]), osolver.D[k]
        d = float(np.abs(a.astype(np.complex128) - b.astype(np.complex128)).max()) if b.size else 0
        scale = float(np.abs(b).max()) if b.size else 0.0
        if dens is not None:
            scale = max(scale, field_floor(osolver, k, dens))
        e = d / scale if scale > 0 else (0.0 if d == 0 else np.inf)
        if verbose and e > 0:
            print(f"{k:>16s} {e:.3e}")
        worst = max(worst, e)
    return worst
