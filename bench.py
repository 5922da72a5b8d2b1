"""Benchmark: electron particle-steps/s of the quasi-cylindrical PSATD PIC
step on one GB300, on the mixed-precision single-run workload -- window
z in [-80, 0], r in [0, 40] (lambda0), Nz=2048, Nr=256, modes m=0,1, 2x1x4
macro-electrons per cell (about 4.2M) in n_e = 2e-3 n_c with a linear
up-ramp over the first 20 lambda0, immobile ions, Gaussian laser a0=3,
w0=10, tau=8 (field FWHM), moving window with injection every 20 steps.
Synthetic seeded plasma (no dataset exists for this workload).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm times the mixed-precision step (the headline `value`: FP32
particles and fields, radial Hankel/derivative GEMMs as BF16x3 products on
the tensor cores) and the plain FP64 step on the same seed through the
public API (Solver / Particles / Frame / PIC_loop), reports their ratio and
the relative deviation of the mixed run's integrated diagnostics from the
FP64 run's, a roofline line for the
dominant kernel, and a CPU baseline (the oracle on the host cores).  The
reference arm times the oracle (the reference's step restated on the CPU,
OpenMP kernels + numpy FFT/GEMM) on all host threads.  N>1 runs independent
replicas, one per GPU (the step does not shard: every transform couples the
whole grid), with the time taken as the maximum over ranks.
"""
import argparse
import copy
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

PEAKS_FILE = os.path.join(HERE, "MEASURED_PEAKS.json")
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}

WORKLOAD = "lpa_mixed_single_run_2048x256_m1"
REFERENCE_STEP_CAP = 20


def workload(seed=0):
    """The mixed-precision single-run LPA configuration."""
    tau = 8.0
    return dict(
        grid_in=dict(Xmin=-80.0, Xmax=0.0, Nx=2048, Rmin=0.0, Rmax=40.0, Nr=256, M=1,
                     DampCells=50),
        eons_in=dict(Nppc=(2, 1, 4), dens=2e-3, charge=-1),
        frame_in=dict(Velocity=1.0, Steps=20),
        laser_in=dict(k0=1.0, a0=3.0, x0=-10.0, Lx=tau / (2 * np.sqrt(np.log(2))), R=10.0,
                      x_foc=-10.0),
        prefill=dict(Xmin=-80.0, Xmax=0.0, Rmin=0.0, Rmax=40.0),
        profiles=[{"coord": "x", "points": [-1e4, -80.0, -60.0, 1e6],
                   "values": [0.0, 0.0, 1.0, 1.0]}],
        seed=seed)


def config_line(cfg):
    g = cfg["grid_in"]
    return {"workload": WORKLOAD, "Nz": g["Nx"], "Nr": g["Nr"], "modes": g["M"] + 1,
            "ppc": list(cfg["eons_in"]["Nppc"]), "dens": cfg["eons_in"]["dens"],
            "a0": cfg["laser_in"]["a0"], "w0": cfg["laser_in"]["R"], "tau": 8.0,
            "window": [g["Xmin"], g["Xmax"], 0.0, g["Rmax"]], "frame_steps": 20,
            "l2": "working set (particles + fields) larger than L2; no flush",
            "parallelism": "replicas"}


# ---------------------------------------------------------------------------
def build_run(cfg, precision, device_index=0, particles_cls=None, **comm_kw):
    """Set the run up through the public API, as the reference's example
    scripts do (examples/lpa_script_small.py:51-95)."""
    from chimeracl_gb300 import Communicator
    from chimeracl_gb300.frame import Frame
    from chimeracl_gb300.laser import add_gausian_pulse
    from chimeracl_gb300.particles import Particles
    from chimeracl_gb300.pic_loop import PIC_loop
    from chimeracl_gb300.solver import Solver

    comm = Communicator(precision=precision, device=device_index, seed=cfg["seed"], **comm_kw)
    solver = Solver(copy.deepcopy(cfg["grid_in"]), comm)
    add_gausian_pulse(solver, dict(cfg["laser_in"]))
    e_in = copy.deepcopy(cfg["eons_in"])
    e_in.update(dx=solver.Args["dx"], dr=solver.Args["dr"], dt=solver.Args["dt"])
    i_in = copy.deepcopy(e_in)
    i_in["charge"] = 1
    i_in["Immobile"] = True
    eons = (particles_cls or Particles)(e_in, comm, seed=cfg["seed"])
    ions = Particles(i_in, comm, seed=cfg["seed"] + 1)
    ions.Args["InjectorSource"] = eons
    eons.make_new_domain(dict(cfg["prefill"]), density_profiles=cfg["profiles"])
    eons.add_new_particles()
    ions.add_new_particles(source=eons)
    eons.free_added()
    f_in = dict(cfg["frame_in"], dt=solver.Args["dt"], DensityProfiles=cfg["profiles"])
    loop = PIC_loop([solver], [eons, ions], [Frame(f_in)], graphs=True)
    return solver, eons, ions, loop


def diagnostics_dev(solver, eons):
    """Integrated diagnostics on the device (float64 reductions): field
    energy sum_m w_m sum (|E|^2 + |B|^2) 2 pi r dr dx over rows r > 0
    (w_0 = 1, w_m = 2); the on-axis longitudinal field |Ex_m0[1, ix]| (x is
    the propagation axis: behind the laser this is the wake); kinetic
    energy sum w (gamma - 1)."""
    import torch
    A, D = solver.Args, solver.DataDev
    r = torch.as_tensor(A["Rgrid"][1:, None], device=D["Ez_m0"].device)
    vol = 2 * np.pi * r * A["dr"] * A["dx"]
    We = torch.zeros((), dtype=torch.float64, device=r.device)
    for m in range(A["M"] + 1):
        wm = 1.0 if m == 0 else 2.0
        for f in ("E", "B"):
            for c in "xyz":
                a = D[f + c + "_m" + str(m)][1:].to(torch.complex128 if m else torch.float64)
                We = We + wm * ((a.abs() ** 2) * vol).sum()
    ex = D["Ex_m0"][1].to(torch.float64).abs()
    # gamma - 1 = p^2 / (1 + gamma) from the momenta, in float64 (1/g_inv - 1
    # cancels: an FP32 g_inv holds nothing of gamma - 1 below 6e-8)
    D = eons.DataDev
    p2 = sum(D[k].to(torch.float64) ** 2 for k in ("px", "py", "pz"))
    kin = (D["w"].to(torch.float64) * p2 / (1.0 + torch.sqrt(1.0 + p2))).sum()
    return We, ex, kin


def field_l2_rel(sol, ref, per_field=None):
    """Pointwise relative L2 difference of all real-space E, B modes (rows
    r > 0) of `sol` against `ref`, in float64 on the device; each field's
    own (E, B and rho per mode) into `per_field` if given."""
    import torch
    A = ref.Args
    num = den = 0.0
    for m in range(A["M"] + 1):
        for k in [f + c + "_m" + str(m) for f in ("E", "B") for c in "xyz"] + ["rho_m" + str(m)]:
            dt = torch.complex128 if m else torch.float64
            a, b = sol.DataDev[k][1:].to(dt), ref.DataDev[k][1:].to(dt)
            dn, dd = float(((a - b).abs() ** 2).sum()), float((b.abs() ** 2).sum())
            if per_field is not None:
                per_field[k] = float(np.sqrt(dn / dd)) if dd > 0 else None
            if k[0] in "EB":
                num += dn
                den += dd
    return float(np.sqrt(num / den))


def compare_runs(cfg, run, ref):
    """Relative differences of `run` against `ref` at the same step: field
    energy, wake amplitude (max on-axis |Ex_m0| behind the laser,
    x < x_laser - 2 Lx), kinetic energy, pointwise field L2."""
    vals = []
    for r in (run, ref):
        We, ex, kin = diagnostics_dev(r["solver"], r["eons"])
        A = r["solver"].Args
        x_las = cfg["laser_in"]["x0"] + r["loop"].it * A["dt"]
        vals.append((float(We), wake_amplitude(ex.cpu().numpy(), A["Xgrid"], x_las,
                                               cfg["laser_in"]["Lx"]), float(kin)))
    (We, wk, kin), (We0, wk0, kin0) = vals
    per = {}
    l2 = field_l2_rel(run["solver"], ref["solver"], per)
    return {"field_energy_rel_err": abs(We / We0 - 1), "wake_ex_rel_err": abs(wk / wk0 - 1),
            "kinetic_rel_err": abs(kin / kin0 - 1), "field_l2_rel_err": l2,
            "field_l2_rel_err_per_field": {k: (None if v is None else float("%.3g" % v))
                                           for k, v in per.items()},
            "at_step": ref["loop"].it}


FULL_RUN_STEPS = 500  # the single run's length


def advance_to(run, n):
    """Step a run (dict of build_run's objects) until its loop reaches step n."""
    while run["loop"].it < n:
        run["loop"].step()


def full_run_accuracy(cfg, device_index=0):
    """The mixed run against the FP64 run on the same seed at the end of the
    full-length run (FULL_RUN_STEPS, fresh runs of the workload), beside
    (a) the FP64 run's own sensitivity there -- the FP64 run with its
    injected coordinates and weights rounded to FP32 (2^-24 relative),
    against the FP64 run: with 2x1x4 particles per cell every radial
    coordinate sits on a grid node, so cell indices and window exits of the
    outermost rows are rounding ties -- and (b) the same comparison with
    2x2x4 particles per cell (no ties)."""
    import torch
    n = FULL_RUN_STEPS

    def fresh(c, prec, particles_cls=None):
        run = dict(zip(("solver", "eons", "ions", "loop"),
                       build_run(c, prec, device_index, particles_cls=particles_cls)))
        advance_to(run, n)
        torch.cuda.synchronize()
        return run

    keys = ("field_energy_rel_err", "wake_ex_rel_err", "kinetic_rel_err", "field_l2_rel_err")
    r64 = fresh(cfg, "fp64")
    r32 = fresh(cfg, "mixed")
    acc = compare_runs(cfg, r32, r64)
    acc["layout"] = "x".join(map(str, cfg["eons_in"]["Nppc"]))
    acc["electrons"] = {"mixed": int(r32["eons"].Args["Np"]), "fp64": int(r64["eons"].Args["Np"])}
    del r32
    alt = fresh(cfg, "fp64", fp32_injected_particles())
    se = compare_runs(cfg, alt, r64)
    acc["fp64_self_sensitivity"] = {k: se[k] for k in keys}
    del alt, r64
    torch.cuda.empty_cache()
    cfg2 = copy.deepcopy(cfg)
    cfg2["eons_in"]["Nppc"] = (2, 2, 4)
    pair = {prec: fresh(cfg2, prec) for prec in ("fp64", "mixed")}
    a2 = compare_runs(cfg2, pair["mixed"], pair["fp64"])
    acc2 = {k: a2[k] for k in keys + ("at_step",)}
    acc2["layout"] = "2x2x4"
    acc2["field_l2_rel_err_per_field"] = a2["field_l2_rel_err_per_field"]
    del pair
    torch.cuda.empty_cache()
    return acc, acc2


def wake_amplitude(ez_row, xgrid, x_laser, Lx):
    sel = xgrid < (x_laser - 2 * Lx)
    return float(np.abs(ez_row[sel]).max()) if sel.any() else float("nan")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
         "utilization.gpu")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 9]
        busy = [r for r in rows if r[9].strip().isdigit() and int(r[9]) >= 50]
        rows = busy or rows  # samples taken under load, when there are any
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------
class Probe:
    """CUDA-event timing of every launch of selected C-ABI calls, with each
    call's algorithmic bytes and flops (counted from its arguments)."""

    def __init__(self, names):
        import torch
        self.torch = torch
        self.names = set(names)
        self.rec = {n: [] for n in names}

    def __call__(self, name, args, fn):
        if name not in self.names:
            return fn()
        t = self.torch
        a, b = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
        a.record()
        r = fn()
        b.record()
        self.rec[name].append((a, b, algorithmic(name, args)))
        return r

    def summary(self):
        self.torch.cuda.synchronize()
        out = {}
        for n, lst in self.rec.items():
            if not lst:
                continue
            ms = [a.elapsed_time(b) for a, b, _ in lst]
            byts = sum(x[2][0] for x in lst)
            flops = sum(x[2][1] for x in lst)
            out[n] = {"launches": len(lst), "ms_total": sum(ms), "bytes": byts, "flops": flops}
        return out


def algorithmic(name, args):
    """(bytes, flops) a call must move/compute at minimum: every operand read
    once and every result written once."""
    if name == "ccl_dht_gemm":
        dtype, batch, m, k, ncols, cplx = args[:6]
        beta = args[13]
        b = 8 if dtype == 0 else 4
        byts = batch * b * (m * k + k * ncols + m * ncols * (2 if beta else 1))
        return byts, batch * 2.0 * m * k * ncols
    if name == "ccl_dht_gemm_batch":
        dtype, batch, m, k, ncols = args[:5]
        beta = args[13]
        b = 8 if dtype == 0 else 4
        byts = sum(b * (m * k + k * n + m * n * (2 if beta else 1)) for n in ncols[:batch])
        return byts, sum(2.0 * m * k * n for n in ncols[:batch])
    if name in ("ccl_fft_forward_batch", "ccl_fft_backward_batch", "ccl_damp_batch"):
        dtype, batch, nrows, nx = args[:4]
        real = args[6] if name == "ccl_fft_forward_batch" else args[7] if \
            name == "ccl_fft_backward_batch" else args[6]
        b = 8 if dtype == 0 else 4
        byts = 0.0
        for e in range(batch):
            rsb = b if real[e] else 2 * b  # real-space side real (mode 0) or complex
            if name == "ccl_damp_batch":  # spectral in + out, real-space row written
                byts += nrows * nx * (2 * 2 * b + rsb)
            else:
                byts += nrows * nx * (2 * b + rsb)
        passes = 2 if name == "ccl_damp_batch" else 1
        return byts, batch * passes * nrows * 5.0 * nx * np.log2(nx)
    if name == "ccl_dht_bf16x3_gemm_batch":
        batch, m, k, ncols = args[:4]
        beta = args[12]
        # FP32 X read, FP32 Y written (read too when accumulating), bf16 hi+lo A
        byts = sum(4 * (m * k + k * n + m * n * (2 if beta else 1)) for n in ncols[:batch])
        return byts, sum(3 * 2.0 * m * k * n for n in ncols[:batch])  # 3 bf16 products
    if name in ("ccl_grad_combine", "ccl_rot_combine"):
        dtype, M, nrows, nx = args[:4]
        b = 8 if dtype == 0 else 4
        per = 5 if name == "ccl_grad_combine" else 9  # complex in + out per cell
        return (M + 1) * nrows * nx * 2 * b * per, 0.0
    if name == "ccl_index_sort":
        dtype, n, Nx, Nr = args[0], args[1], args[5], args[8]
        b = 8 if dtype == 0 else 4
        C = (Nx - 1) * (Nr - 1)
        # x, y, z read; key and sort index written; counts and offsets written
        return n * (3 * b + 4 + 4) + (C + 1) * 4 + (C + 2) * 4, 0.0
    if name in ("ccl_gather_push", "ccl_gather_push_cells", "ccl_gather_push_cells_lo"):
        dtype, M, n = args[0], args[1], args[2]
        Nx, Nr = (args[13], args[16]) if name == "ccl_gather_push" else (args[14], args[17])
        b = 8 if dtype == 0 else 4
        lo = 3 * b if name.endswith("_lo") else 0
        # x, y, z (+ low parts), u, g_inv read, u, g_inv written, sort index;
        # E, B read once
        return n * (7 * b + lo + 4 * b + 4) + 6 * (2 * M + 1) * Nx * Nr * b, 0.0
    if name == "ccl_push_x_keys":
        dtype, n, Nx, Nr = args[0], args[1], args[13], args[16]
        b = 8 if dtype == 0 else 4
        lo = 6 * b if args[5] else 0  # low parts read and written
        C = (Nx - 1) * (Nr - 1)
        # x, y, z, px, py, pz, g_inv read, x, y, z and the key written; counts
        return n * (10 * b + lo + 4) + (C + 1) * 4, 0.0
    if name == "ccl_index_sort_keyed":
        n, Nx, Nr = args[0], args[1], args[2]
        C = (Nx - 1) * (Nr - 1)
        # key read, sort index written; counts read, offsets written
        return n * (4 + 4) + (C + 1) * 4 + (C + 2) * 4, 0.0
    if name == "ccl_psatd_advance_split":
        dtype, n = args[0], args[1]
        b = 8 if dtype == 0 else 4
        # 8 coefficients + 6 complex fields + 3 sources read, 6 complex written
        return n * (8 + (6 + 3) * 2 + 6 * 2) * b, 0.0
    if name == "ccl_psatd_advance":
        dtype, n = args[0], args[1]
        b = 8 if dtype == 0 else 4
        # 15 complex + 3 real read, 6 complex written per spectral cell
        return n * (15 * 2 + 3 + 6 * 2) * b, 0.0
    return 0, 0.0


def install_probe(probe):
    from chimeracl_gb300 import _lib
    orig = _lib.call

    def call(name, *args):
        return probe(name, args, lambda: orig(name, *args))
    _lib.call = call
    for mod in list(sys.modules.values()):
        if getattr(mod, "__name__", "").startswith("chimeracl_gb300") and hasattr(mod, "call") \
                and getattr(mod, "call") is orig:
            mod.call = call
    return orig


def remove_probe(orig):
    from chimeracl_gb300 import _lib
    for mod in list(sys.modules.values()):
        if getattr(mod, "__name__", "").startswith("chimeracl_gb300") and hasattr(mod, "call"):
            mod.call = orig
    _lib.call = orig


# ---------------------------------------------------------------------------
def time_arm(cfg, precision, steps, warmup, device_index, dist):
    """Warm up, then time exactly `steps` steps (barrier + synchronize on both
    sides, CUDA events on the step stream)."""
    import torch
    from chimeracl_gb300 import _lib
    solver, eons, ions, loop = build_run(cfg, precision, device_index)
    for _ in range(warmup):
        loop.step()
    torch.cuda.synchronize()
    np_sum = 0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = _lib.launch_count()
    c0, r0 = loop.graph_kernels_captured, loop.graph_kernels_replayed
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(device_index) as clk:
        time.sleep(0.3)  # let the sampler start before the timed region
        e0.record()
        for _ in range(steps):
            np_sum += eons.Args["Np"]
            loop.step()
        e1.record()
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    # library kernels that ran: launched eagerly, or replayed from a graph
    launches = (_lib.launch_count() - n0 - (loop.graph_kernels_captured - c0)
                + (loop.graph_kernels_replayed - r0))
    return dict(solver=solver, eons=eons, ions=ions, loop=loop, ms=ms, np_sum=np_sum,
                launches=launches, clocks=clk.summary())


def e2e_arm(run, steps):
    """The same steps through PIC_loop.step() timed on the host clock, with
    each step's injector draws generated on the host and uploaded (the H2D
    traffic of make_new_domain at window shifts) and each step's result -- the
    on-axis Ez line, the wake diagnostic -- copied to pinned host memory and
    read on the host.  The copies are pipelined: step k's line is read (its
    peak |Ez| taken) while step k + 1 runs, through two pinned buffers and
    an event per copy; the clock stops after the last line is read."""
    import torch
    solver, eons, loop = run["solver"], run["eons"], run["loop"]
    comm = solver.comm
    ez = solver.DataDev["Ez_m0"]
    host = [torch.empty(ez.shape[-1] * (2 if ez.is_complex() else 1),
                        dtype=torch.float32 if ez.dtype in (torch.float32, torch.complex64)
                        else torch.float64).pin_memory() for _ in range(2)]
    ev = [torch.cuda.Event(), torch.cuda.Event()]
    peaks = []

    def read(k):  # the host side of step k's result
        ev[k % 2].synchronize()
        # numpy on the host (torch's CPU kernels would wake its thread pool)
        peaks.append(float(np.abs(host[k % 2].numpy()).max()))
        comm.d2h_bytes += host[k % 2].numel() * host[k % 2].element_size()

    line0 = torch.view_as_real(ez[1]).reshape(-1) if ez.is_complex() else ez[1]
    host[0].copy_(line0)  # first use of the copy path outside the timed region
    torch.cuda.synchronize()
    h0, d0 = comm.h2d_bytes, comm.d2h_bytes
    np_sum = 0
    t0 = time.perf_counter()
    for k in range(steps):
        np_sum += eons.Args["Np"]
        loop.step()
        line = solver.DataDev["Ez_m0"][1]
        line = torch.view_as_real(line).reshape(-1) if line.is_complex() else line
        host[k % 2].copy_(line, non_blocking=True)
        ev[k % 2].record()
        if k > 0:
            read(k - 1)
    if steps:
        read(steps - 1)
    t = time.perf_counter() - t0
    assert len(peaks) == steps and all(np.isfinite(peaks))
    return dict(s=t, np_sum=np_sum, h2d=(comm.h2d_bytes - h0) / steps,
                d2h=(comm.d2h_bytes - d0) / steps)


def _oracle_rate_here(cfg, steps, warmup):
    """Time the oracle in this process (see cpu_oracle_rate), its FFTs on all
    host threads."""
    from oracle import pic_oracle as po
    from oracle.kernels import PortKernels
    po.use_threaded_fft(-1)
    K = PortKernels()
    s, e, i, loop = po.build_lpa(copy.deepcopy(cfg["grid_in"]), cfg["eons_in"], cfg["frame_in"],
                                 cfg["laser_in"], prefill=cfg["prefill"], K=K, seed=cfg["seed"],
                                 density_profiles=cfg["profiles"])
    for _ in range(warmup):
        loop.step()
    n = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        n += e.Args["Np"]
        loop.step()
    t = time.perf_counter() - t0
    return n / t, K.num_threads(), t


def cpu_oracle_rate(cfg, steps, warmup=1):
    """The oracle (reference step restated; C kernels with OpenMP over the
    host cores, numpy FFT and GEMM) on the same workload: electron
    particle-steps/s over `steps` steps after `warmup`, the thread count,
    the seconds.  The oracle's FFTs run on all host threads (scipy.fft) as
    its kernels (OpenMP) and GEMMs (BLAS) do.

    It runs in a child process without torch, with OMP_WAIT_POLICY=passive:
    OpenMP worker threads that spin between the oracle's short kernels
    compete with numpy's BLAS threads for the cores (measured: 1.4x slower
    on the 2048 x 256 workload, 12x on 512 x 64), and once a library has
    started OpenMP in a process the policy can no longer be set."""
    env = dict(os.environ, OMP_WAIT_POLICY="passive")
    code = ("import json, sys; sys.path.insert(0, %r); import bench; "
            "cfg = json.load(sys.stdin); "
            "print(json.dumps(bench._oracle_rate_here(cfg, %d, %d)))" % (HERE, steps, warmup))
    r = subprocess.run([sys.executable, "-c", code], input=json.dumps(cfg), env=env, cwd=HERE,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CPU oracle run failed:\n" + r.stderr[-2000:])
    rate, cores, t = json.loads(r.stdout.strip().splitlines()[-1])
    return rate, cores, t


def load_peaks():
    try:
        with open(PEAKS_FILE) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return dict(FALLBACK_PEAKS), "fallback"


# DRAM bytes (read + write) per call of the 2048 x 256, M = 1 workload, summed
# over the call's kernels in one ncu capture.  ccl_index_sort:
#   ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum
#       --clock-control none --nvtx --nvtx-include "prof/" <one sort of the workload>
# ccl_index_sort_keyed (k_scan_lookback 2.1 MB + k_scatter 20.8 MB +
# k_cell_fixup 2.0 MB, the sort_indx the scatter writes staying in L2):
#   profiles/sort_and_combine_kernels_mixed_2048x256_ncu_full.md
MEASURED_TRAFFIC = {"ccl_index_sort": 86.7e6, "ccl_index_sort_keyed": 24.9e6}


def roofline(probe_summary, peaks, src):
    """Roofline line of the kernel with the largest share of the probed
    time: achieved = algorithmic bytes (or flops) per launch / mean launch
    time; the tensor-core GEMM is checked against both the HBM copy peak and
    the bf16 tensor peak and reported against the one it is closer to."""
    if not probe_summary:
        return None
    name, s = max(probe_summary.items(), key=lambda kv: kv[1]["ms_total"])
    per_s = s["ms_total"] / s["launches"] * 1e-3
    gbs = s["bytes"] / s["launches"] / per_s / 1e9
    line = {"kernel": name, "launches": s["launches"], "ms_per_launch": round(per_s * 1e3, 5),
            "traffic": MEASURED_TRAFFIC.get(name), "peak_source": src}
    hbm = {"bound": "hbm", "achieved": round(gbs, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
           "frac": round(gbs / peaks["hbm_gbs"], 4)}
    if name == "ccl_dht_bf16x3_gemm_batch":
        tfs = s["flops"] / s["launches"] / per_s / 1e12
        pk = peaks.get("bf16_tflops", FALLBACK_PEAKS["bf16_tflops"])
        ten = {"bound": "tensor", "achieved": round(tfs, 2), "peak": pk, "unit": "TFLOP/s",
               "frac": round(tfs / pk, 4)}
        line.update(ten if ten["frac"] > hbm["frac"] else hbm)
        line["hbm_frac"], line["tensor_frac"] = hbm["frac"], ten["frac"]
    else:
        line.update(hbm)
    return line


# ---------------------------------------------------------------------------
def init_dist(ngpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return None, 0, 0, 1
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return dist, rank, local, world


def reduce_max(dist, value, device):
    """Maximum of a float over ranks."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, value, device):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_reference(args):
    dist, rank, local, world = init_dist(args.gpus)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    cfg = workload(seed=1000)
    # a bounded sample: at most REFERENCE_STEP_CAP oracle steps (about 1 s
    # each on this workload), so the arm ends within a few minutes for any
    # --steps; one window shift falls inside a sample of 20
    n = max(1, min(args.steps, REFERENCE_STEP_CAP))
    rate, cores, t = cpu_oracle_rate(cfg, steps=n, warmup=min(args.warmup, 1))
    line = {"metric": "electron particle-steps/s", "value": rate, "unit": "particle-steps/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "steps_timed": n,
            "ms_per_step": 1e3 * t / n, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded plasma, laser)",
            "config": config_line(cfg),
            "cpu_baseline": {"value": rate, "unit": "particle-steps/s", "cores": cores,
                             "kind": "port",
                             "sample": f"{n} steps of the workload (of {args.steps} "
                                       f"requested) after {min(args.warmup, 1)} warm-up"},
            "e2e": {"value": rate, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def run_ours(args):
    import torch
    dist, rank, local, world = init_dist(args.gpus)
    dev = torch.device("cuda", local)
    cfg = workload(seed=1000 + rank)
    # mixed form (headline) and the plain FP64 form on the same seed
    r32 = time_arm(cfg, "mixed", args.steps, args.warmup, local, dist)
    diagnostics_dev(r32["solver"], r32["eons"])  # first use of torch's reductions
    e2e = e2e_arm(r32, args.steps)
    probe = Probe(["ccl_dht_bf16x3_gemm_batch", "ccl_grad_combine", "ccl_rot_combine",
                   "ccl_dht_gemm_batch", "ccl_dht_gemm", "ccl_fft_forward_batch",
                   "ccl_fft_backward_batch", "ccl_damp_batch", "ccl_index_sort",
                   "ccl_push_x_keys", "ccl_index_sort_keyed", "ccl_deposit_vector",
                   "ccl_deposit_scalar", "ccl_gather_push", "ccl_gather_push_cells",
                   "ccl_gather_push_cells_lo", "ccl_psatd_advance",
                   "ccl_psatd_advance_split"])
    orig = install_probe(probe)
    r32["loop"].graphs = False  # the probe times each launch: run the steps eagerly
    for _ in range(min(args.steps, 5)):
        r32["loop"].step()
    r32["loop"].graphs = True
    remove_probe(orig)
    prof = probe.summary()
    r64 = time_arm(cfg, "fp64", args.steps, args.warmup, local, dist)
    # accuracy of the mixed run vs the FP64 run at the end of the full run
    # (untimed: both runs are stepped on to the workload's 500 steps)
    acc, acc2 = ({}, {}) if args.no_accuracy else full_run_accuracy(cfg, local)
    ms32 = reduce_max(dist, r32["ms"], dev)
    ms64 = reduce_max(dist, r64["ms"], dev)
    np32 = reduce_sum(dist, r32["np_sum"], dev)
    np64 = reduce_sum(dist, r64["np_sum"], dev)
    e2e_s = reduce_max(dist, e2e["s"], dev)
    e2e_np = reduce_sum(dist, e2e["np_sum"], dev)
    value = np32 / (ms32 * 1e-3)
    v64 = np64 / (ms64 * 1e-3)
    if rank == 0:
        peaks, src = load_peaks()
        line = {
            "metric": "electron particle-steps/s", "value": value, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms32 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+bf16x3", "data": "synthetic (seeded plasma, laser)",
            "config": config_line(cfg),
            "fp64": {"value": v64, "ms_per_step": ms64 / args.steps, "dtype": "f64",
                     "gpu_launches": r64["launches"]},
            "mixed_over_fp64": value / v64,
            "mixed_vs_fp64_error": acc,
            "mixed_vs_fp64_error_2x2x4": acc2,
            "e2e": {"value": e2e_np / e2e_s, "unit": "particle-steps/s",
                    "h2d_bytes_per_step": int(e2e["h2d"]), "d2h_bytes_per_step": int(e2e["d2h"])},
            "gpu_launches": r32["launches"],
            "graph_replays": r32["loop"].graph_replays,
            "clocks": r32["clocks"],
            "roofline": roofline(prof, peaks, src),
            "kernel_probe": {k: {"launches": v["launches"], "ms_total": round(v["ms_total"], 4)}
                             for k, v in prof.items()},
        }
        if world == 1 and not args.no_extra_workloads:
            # the large-mode and batched workloads, with few steps each, and
            # the differentiable run's adjoint
            line["large_modes"] = large_modes_line(min(args.steps, 10), 3, args.batch_seed)
            line["batched"] = batched_line(args.batch_runs, min(args.steps, 20), 3,
                                           args.batch_seed)
            line["adjoint"] = adjoint_line()
        if world == 1 and not args.no_cpu_baseline:
            rate, cores, t = cpu_oracle_rate(cfg, steps=args.cpu_steps, warmup=1)
            line["cpu_baseline"] = {"value": rate, "unit": "particle-steps/s", "cores": cores,
                                    "kind": "port",
                                    "sample": f"{args.cpu_steps} FP64 steps of the workload "
                                              "after 1 warm-up step (oracle, OpenMP + numpy)"}
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


LARGE_MODES_WORKLOAD = "lpa_large_modes_4096x512_m2"


def large_modes_workload(seed=0):
    """The large-mode run: Nz = 4096, Nr = 512 on the single run's cells
    (window z in [-160, 0], r in [0, 80] lambda0), modes m = 0, 1, 2, 2x2x4
    macro-electrons per cell (about 33.5M) in uniform n_e = 1e-3 n_c,
    immobile ions, laser a0 = 4, w0 = 12, tau = 10 (field FWHM) centred and
    focused at z = -20 (its envelope is 1.5e-5 of the peak at the window's
    front), with a 20% m = 2 astigmatic term; moving window with injection
    every 20 steps; seeded."""
    tau = 10.0
    return dict(
        grid_in=dict(Xmin=-160.0, Xmax=0.0, Nx=4096, Rmin=0.0, Rmax=80.0, Nr=512, M=2,
                     DampCells=50),
        eons_in=dict(Nppc=(2, 2, 4), dens=1e-3, charge=-1),
        frame_in=dict(Velocity=1.0, Steps=20),
        laser_in=dict(k0=1.0, a0=4.0, x0=-20.0, Lx=tau / (2 * np.sqrt(np.log(2))), R=12.0,
                      x_foc=-20.0, astig=0.2),
        prefill=dict(Xmin=-160.0, Xmax=0.0, Rmin=0.0, Rmax=80.0),
        profiles=None, seed=seed)


def run_large_modes(args):
    print(json.dumps(large_modes_line(args.steps, args.warmup, args.batch_seed)))
    return 0


def large_modes_line(steps, warmup, seed):
    """The large-mode run in the mixed form and in FP64 on the same seed:
    device-timed steps of each (CUDA events, after the warm-up) and the
    mixed run's relative error against the FP64 run per field (E, B, rho of
    each mode, pointwise L2) and in the integrated diagnostics at the same
    step."""
    import torch

    class _A:
        pass
    args = _A()
    args.steps, args.warmup = steps, warmup
    cfg = large_modes_workload(seed=seed)
    r32 = time_arm(cfg, "mixed", args.steps, args.warmup, 0, None)
    r64 = time_arm(cfg, "fp64", args.steps, args.warmup, 0, None)
    torch.cuda.synchronize()
    g = cfg["grid_in"]
    line = {
        "metric": "electron particle-steps/s (large-mode run)",
        "value": r32["np_sum"] / (r32["ms"] * 1e-3), "unit": "particle-steps/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r32["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+bf16x3",
        "data": "synthetic (seeded plasma, laser)",
        "config": {"workload": LARGE_MODES_WORKLOAD, "Nz": g["Nx"], "Nr": g["Nr"],
                   "modes": g["M"] + 1, "ppc": [2, 2, 4], "a0": 4.0, "w0": 12.0, "tau": 10.0,
                   "astig": 0.2, "l2": "working set larger than L2; no flush"},
        "fp64": {"value": r64["np_sum"] / (r64["ms"] * 1e-3),
                 "ms_per_step": r64["ms"] / args.steps},
        "mixed_over_fp64": (r32["np_sum"] / r32["ms"]) / (r64["np_sum"] / r64["ms"]),
        "mixed_vs_fp64_error": compare_runs(cfg, r32, r64),
        "gpu_launches": r32["launches"],
        "clocks": r32["clocks"],
    }
    del r32, r64
    torch.cuda.empty_cache()
    return line


BATCHED_WORKLOAD = "lpa_batched_uneven_64"


def batched_cases(n=64, seed=0):
    """The batched small-run workload: n independent LPA runs with Nz drawn
    from {256, 384, 512, 768, 1024} and Nr from {32, 64, 96, 128}, m = 0, 1,
    1x1x4 macro-electrons per cell, n_e in [5e-4, 3e-3] n_c, laser a0 in
    [1, 3] and w0 in [4, 10] lambda0 (tau = 5, centred and focused at
    z = -12), on the 512 x 64 run's cells (dz = 40/512, dr = 20/64), moving
    window with injection every 20 steps, absorbing edges of min(50, Nz/16)
    cells (the damping profile is below 1 over 4/3 of them at either end;
    the pulse, +-2 Lx around its centre, stays clear of both); seeded."""
    rng = np.random.default_rng(seed)
    dx, dr = 40.0 / 512, 20.0 / 64
    cases = []
    for i in range(n):
        nx = int(rng.choice([256, 384, 512, 768, 1024]))
        nr = int(rng.choice([32, 64, 96, 128]))
        dens, a0, w0 = (float(rng.uniform(*b)) for b in ((5e-4, 3e-3), (1.0, 3.0), (4.0, 10.0)))
        win = dict(Xmin=-nx * dx, Xmax=0.0, Rmin=0.0, Rmax=nr * dr)
        cases.append(dict(
            grid_in=dict(win, Nx=nx, Nr=nr, M=1, DampCells=min(50, nx // 16)),
            eons_in=dict(Nppc=(1, 1, 4), dens=dens, charge=-1),
            frame_in=dict(Velocity=1.0, Steps=20),
            laser_in=dict(k0=1.0, a0=a0, x0=-12.0, Lx=5.0 / (2 * np.sqrt(np.log(2))), R=w0,
                          x_foc=-12.0),
            prefill=dict(win), profiles=None, seed=seed * 1000 + i))
    return cases


def run_batched(args):
    print(json.dumps(batched_line(args.batch_runs, args.steps, args.warmup, args.batch_seed)))
    return 0


def batched_line(nruns, steps, warmup, seed):
    """Aggregate electron particle-steps/s of the batched workload through
    PIC_batch in both of its modes -- each run's step on its own stream, and
    the whole batch step as one CUDA graph -- with the lane count picked by
    its autotuner during the warm-up; `value` is the faster mode's, beside
    the same runs stepped one by one on one stream."""
    import torch
    from chimeracl_gb300.batch import PIC_batch
    from chimeracl_gb300 import _lib
    class _A:
        pass
    args = _A()
    args.steps, args.warmup = steps, warmup
    cases = batched_cases(nruns, seed=seed)
    runs = [build_run(c, "mixed") for c in cases]
    loops = [r[3] for r in runs]

    def tuned(one_graph):
        bt = PIC_batch(loops, one_graph=one_graph)
        while bt.lanes is None and bt.it < 200:  # tuning, then the warm-up proper
            bt.step()
        for _ in range(args.warmup):
            bt.step()
        torch.cuda.synchronize()
        return bt

    def kernels_run(bts):
        # library kernels launched eagerly or replayed from graphs (the
        # loops' own graphs and the batches' one-graph captures)
        objs = list(loops) + list(bts)
        return (_lib.launch_count()
                - sum(o.graph_kernels_captured for o in objs)
                + sum(o.graph_kernels_replayed for o in objs))

    def timed(fn, bts=()):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        n0 = kernels_run(bts)
        with ClockSampler(0) as clk:
            time.sleep(0.3)
            e0.record()
            np_sum = fn()
            e1.record()
            torch.cuda.synchronize()
        return np_sum, e0.elapsed_time(e1), kernels_run(bts) - n0, clk.summary()

    def batched(bt):
        def fn():
            np_sum = 0
            for _ in range(args.steps):
                np_sum += bt.electrons()
                bt.step()
            return np_sum
        return fn

    def alone():
        np_sum = 0
        for lp in loops:
            for _ in range(args.steps):
                np_sum += int(lp.species[0].Args["Np"])
                lp.step()
        return np_sum

    # each run's step on its own stream (three graph replays per run), then
    # the whole batch step as one graph, then the runs one by one
    b = tuned(False)
    nb, msb, lb, clk = timed(batched(b), [b])
    bg = tuned(True)
    ng, msg, lg, _ = timed(batched(bg), [bg])
    n1, ms1, l1, _ = timed(alone)
    modes = {"streams": (nb, msb, b, lb), "one_graph": (ng, msg, bg, lg)}
    best = max(modes, key=lambda m: modes[m][0] / modes[m][1])
    nb, msb, b, lb = modes[best]
    line = {
        "metric": "electron particle-steps/s (batched runs)", "value": nb / (msb * 1e-3),
        "unit": "particle-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": msb / args.steps, "higher_is_better": True, "scaling": "weak",
        "batch_mode": best,
        "batch_modes": {m: {"value": v[0] / (v[1] * 1e-3), "ms_per_step": v[1] / args.steps,
                            "lanes": v[2].lanes} for m, v in modes.items()},
        "vs_baseline": None, "dtype": "f32+bf16x3", "data": "synthetic (seeded plasma, lasers)",
        "config": {"workload": BATCHED_WORKLOAD, "runs": len(runs),
                   "grids": sorted({(c["grid_in"]["Nx"], c["grid_in"]["Nr"]) for c in cases}),
                   "ppc": [1, 1, 4], "modes": 2, "frame_steps": 20,
                   "l2": "working set larger than L2; no flush"},
        "lanes": b.lanes,
        "lane_tuning_ms": {str(c): round(1e3 * statistics.median(v), 3)
                           for c, v in b.tune_log.items() if v},
        "one_by_one": {"value": n1 / (ms1 * 1e-3), "ms_per_step": ms1 / args.steps},
        "batched_over_one_by_one": (nb / msb) / (n1 / ms1),
        "one_graph_replays": bg.graph_replays,
        "gpu_launches": lb,
        "clocks": clk,
    }
    del runs, loops, b, bg, modes
    torch.cuda.empty_cache()
    return line


ADJOINT_WORKLOAD = "lpa_differentiable_1024x128_100steps"


def adjoint_line(seed=0, nsteps=100, every=10, precision="mixed"):
    """The differentiable run (1024 x 128 on the 512 x 64 run's window, m =
    0, 1, 2x2x4 per cell, a0 = 2 laser, 32 density knots, 100 steps): the
    plain forward step (graph replays, no checkpoints) against the adjoint:
    the forward with a checkpoint every `every` steps and the reverse sweep
    (each segment recomputed from its checkpoint, then stepped backwards),
    per step; the gradients of the wake loss w.r.t. (a0, w0, x_foc)."""
    import torch
    from chimeracl_gb300.adjoint import build_problem_run, differentiable_problem
    problem, params, knots = differentiable_problem(seed=seed, nsteps=nsteps, every=every,
                                                    precision=precision)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    # the plain forward: warm-up, then the rest of the run timed
    run = build_problem_run(problem, params, knots)
    warm = 3
    for _ in range(warm):
        run["loop"].step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(nsteps - warm):
        run["loop"].step()
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / (nsteps - warm)
    del run
    # forward with checkpoints, then the reverse sweep (twice: the first
    # builds the library's lazily created tables and the reverse step's
    # graphs' first captures; the second is timed)
    run = build_problem_run(problem, params, knots)
    adj = run["adjoint"]
    _, t_fwd = timed(lambda: adj.run(nsteps))
    loss = float(adj.wake_loss(problem["loss_width"]))
    adj.gradients(problem["loss_width"])
    (g_laser, g_knots), t_bwd = timed(lambda: adj.gradients(problem["loss_width"]))
    adj.profile_phases = True
    adj.gradients(problem["loss_width"])
    phases = {k: round(1e3 * v / nsteps, 4) for k, v in adj.timing.items()}
    line = {"workload": ADJOINT_WORKLOAD, "precision": precision, "steps": nsteps,
            "checkpoint_every": every, "loss": loss,
            "forward_ms_per_step": fwd_ms,
            "forward_with_checkpoints_ms_per_step": 1e3 * t_fwd / nsteps,
            "adjoint_ms_per_step": 1e3 * t_bwd / nsteps,
            "adjoint_over_forward": (1e3 * t_bwd / nsteps) / fwd_ms,
            "adjoint_phases_ms_per_step": phases,
            "grad_a0_w0_xfoc": [float(v) for v in g_laser],
            "grad_knots_max": float(np.abs(g_knots).max())}
    del run, adj
    torch.cuda.empty_cache()
    return line


def fp32_injected_particles():
    """Particles (FP64) whose injector output -- coordinates and weights of
    every prefilled or injected particle -- is rounded through FP32: the
    particles an FP32 run starts from, stepped in FP64.  The reference for
    the step error of the FP32 forms on the same initial particles."""
    from chimeracl_gb300.particles import Particles

    class Fp32InjectedParticles(Particles):
        def make_new_domain(self, parts_in, density_profiles=None):
            super().make_new_domain(parts_in, density_profiles)
            for k in ("x_new", "y_new", "z_new", "w_new"):
                t = self.DataDev[k]
                t.copy_(t.float().double())

    return Fp32InjectedParticles


def run_accuracy(args):
    """The mixed form against FP64 after `acc_steps` steps, on the bench
    workload (2x1x4 particles per cell: every radial position on a grid
    node) and with 2x2x4 per cell (none on a node): against the FP64 run on
    the same seed, and against the FP64 run on the same FP32-rounded
    particles (the step error alone); and the mixed form with compensated
    coordinates (FP64-exact injection, cell-relative fractions) against the
    FP64 run on the same seed."""
    import torch
    out = {}
    for name, nppc in (("2x1x4", None), ("2x2x4", (2, 2, 4))):
        cfg = workload()
        if nppc:
            cfg["eons_in"]["Nppc"] = nppc
        runs = {}
        for tag, prec, cls, kw in (
                ("fp64", "fp64", None, {}),
                ("fp64_fp32_particles", "fp64", fp32_injected_particles(), {}),
                ("mixed", "mixed", None, {}),
                ("mixed_compensated", "mixed", None, {"compensated_positions": True})):
            solver, eons, ions, loop = build_run(cfg, prec, particles_cls=cls, **kw)
            for _ in range(args.acc_steps):
                loop.step()
            torch.cuda.synchronize()
            runs[tag] = dict(solver=solver, eons=eons, ions=ions, loop=loop)
        out[name] = {
            "mixed_vs_fp64": compare_runs(cfg, runs["mixed"], runs["fp64"]),
            "mixed_vs_fp64_same_particles": compare_runs(cfg, runs["mixed"],
                                                         runs["fp64_fp32_particles"]),
            "fp64_same_particles_vs_fp64": compare_runs(cfg, runs["fp64_fp32_particles"],
                                                        runs["fp64"]),
            "mixed_compensated_vs_fp64": compare_runs(cfg, runs["mixed_compensated"],
                                                      runs["fp64"]),
            "electrons": {k: int(r["eons"].Args["Np"]) for k, r in runs.items()}}
        del runs
        torch.cuda.empty_cache()
    print(json.dumps({"accuracy": out, "steps": args.acc_steps, "workload": WORKLOAD}))
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the full-length mixed-vs-FP64 comparison")
    ap.add_argument("--no-extra-workloads", action="store_true",
                    help="skip the large-mode and batched lines of the default run")
    ap.add_argument("--accuracy", action="store_true",
                    help="run the mixed-vs-FP64 accuracy study instead of the benchmark")
    ap.add_argument("--acc-steps", type=int, default=608)
    ap.add_argument("--workload", default="single",
                    choices=["single", "batched", "large_modes", "adjoint"],
                    help="batched: 64 small uneven runs through PIC_batch; large_modes: "
                         "the 4096 x 512, m = 0..2 run, mixed against FP64 (1 GPU); "
                         "adjoint: the differentiable run's forward and reverse sweep")
    ap.add_argument("--adj-steps", type=int, default=100,
                    help="steps of the differentiable run (--workload adjoint)")
    ap.add_argument("--batch-runs", type=int, default=64)
    ap.add_argument("--batch-seed", type=int, default=0)
    args = ap.parse_args(argv)
    if args.warmup < 3 and args.impl == "ours":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    if args.accuracy:
        return run_accuracy(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "large_modes":
        return run_large_modes(args)
    if args.workload == "adjoint":
        print(json.dumps(adjoint_line(nsteps=args.adj_steps)))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
