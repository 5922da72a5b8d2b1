"""Generate the golden fixtures of tests/golden/ from the reference's own
OpenCL kernels (compiled unchanged as C++ into oracle/_ref) driven by the
oracle's host restatement of the reference step.

    python -m tests.golden.make_golden [name.npz ...]   # needs oracle/_ref built

Each case is a small moving-window LPA run (prefilled plasma, immobile ions,
Gaussian laser, frame shift + injection every `steps` steps) stopped after
`nsteps` steps; the fixture holds the sort arrays ("key:" entries, exact),
the real-space and spectral fields and the electron arrays."""
import copy
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    "lpa_m1_64x16.npz": dict(Nx=64, Nr=16, M=1, steps=2, nsteps=3, seed=21),
    "lpa_m0_64x16.npz": dict(Nx=64, Nr=16, M=0, steps=2, nsteps=3, seed=22),
}

# full runs: the 512 x 64, M = 1 LPA configuration (a0 = 2 laser, 2x2x4
# macro-electrons per cell, moving window with injection every 20 steps)
# for 200 steps; the fixture keeps summaries (integrated diagnostics,
# counts, the final cell offsets and on-axis field rows), not the 0.5M
# particles
FULL_RUNS = {
    "lpa_m1_512x64_200steps.npz": dict(Nx=512, Nr=64, M=1, nsteps=200, seed=21),
}

# the 2048 x 256, M = 1 single run (2x1x4 per cell, density up-ramp over the
# window's first 20 lambda0, a0 = 3 laser), 3 steps from its first injection;
# and the same run with 2x2x4 per cell (no particle on a grid node: with one
# radial particle per cell every radius is a rounding tie between two cells,
# which the injector's last-bit sin/cos rounding decides)
BENCH_RUNS = {
    "lpa_m1_2048x256_3steps.npz": dict(nsteps=3, seed=1000),
    "lpa_m1_2048x256_2x2x4_3steps.npz": dict(nsteps=3, seed=1000, nppc=(2, 2, 4)),
}

# further grid shapes: 1024 x 128 on the 512 x 64 run's window (the
# differentiable run's grid, FP64 forward) for 20 steps, and the 384 x 96
# run of the batched workload (1x1x4 per cell, entry 6 of its 64 seeded
# runs) for 30 steps
SHAPE_RUNS = {
    "lpa_m1_1024x128_20steps.npz": dict(kind="window", Nx=1024, Nr=128, M=1, nsteps=20,
                                        seed=31),
    "lpa_m1_384x96_30steps.npz": dict(kind="batched", index=6, nsteps=30, seed=0),
}


def golden_run(name):
    """(case, cfg or None) of a full-run fixture by file name."""
    if name in FULL_RUNS:
        return FULL_RUNS[name], None
    if name in BENCH_RUNS:
        return BENCH_RUNS[name], bench_cfg(BENCH_RUNS[name])
    case = SHAPE_RUNS[name]
    if case["kind"] == "window":
        from tests.lpa_setup import small_lpa
        return case, small_lpa(Nx=case["Nx"], Nr=case["Nr"], M=case["M"], seed=case["seed"])
    import bench
    return case, bench.batched_cases(64, seed=case["seed"])[case["index"]]

FIELDS = ("rho", "Jx", "Jz", "Ex", "Ez", "By", "Bz")


def case_cfg(case):
    from tests.lpa_setup import small_lpa
    return small_lpa(Nx=case["Nx"], Nr=case["Nr"], M=case["M"], steps=case["steps"],
                     seed=case["seed"], damp=6)


def collect(solver, eons):
    st = {}
    M = solver.Args["M"] if hasattr(solver, "Args") else 0
    D = solver.D if hasattr(solver, "D") else solver.DataDev
    for f in FIELDS:
        for m in range(M + 1):
            st[f"{f}_m{m}"] = np.asarray(D[f"{f}_m{m}"])
            if f != "rho":
                st[f"{f}_fb_m{m}"] = np.asarray(D[f"{f}_fb_m{m}"])
    E = eons.D if hasattr(eons, "D") else eons.DataDev
    for k in ("x", "y", "z", "px", "py", "pz", "g_inv", "w"):
        st["p:" + k] = np.asarray(E[k])
    for k in ("indx_in_cell", "sum_in_cell", "cell_offset", "sort_indx"):
        st["key:" + k] = np.asarray(E[k]).astype(np.uint32)
    return st


def run_case(case, K):
    from oracle import pic_oracle as po
    cfg = case_cfg(case)
    s, e, i, loop = po.build_lpa(copy.deepcopy(cfg["grid_in"]), cfg["eons_in"], cfg["frame_in"],
                                 cfg["laser_in"], prefill=cfg["prefill"], K=K, seed=cfg["seed"])
    for _ in range(case["nsteps"]):
        loop.step()
    return collect(s, e)


def run_full(case, K, cfg=None):
    """A full run (FULL_RUNS, or BENCH_RUNS with the benchmark's `cfg`)
    through the oracle host with kernel set K; returns its summary arrays."""
    from oracle import pic_oracle as po
    from tests.lpa_setup import small_lpa
    if cfg is None:
        cfg = small_lpa(Nx=case["Nx"], Nr=case["Nr"], M=case["M"], seed=case["seed"])
    s, e, i, loop = po.build_lpa(copy.deepcopy(cfg["grid_in"]), cfg["eons_in"], cfg["frame_in"],
                                 cfg["laser_in"], prefill=cfg["prefill"], K=K, seed=cfg["seed"],
                                 density_profiles=cfg.get("profiles"))
    for _ in range(case["nsteps"]):
        loop.step()
    d = po.diagnostics(s, [e])
    st = {"diag:" + k: np.float64(v) for k, v in d.items()}
    st["count:Np"] = np.int64(e.Args["Np"])
    st["count:Np_stay"] = np.int64(e.Args["Np_stay"])
    st["key:cell_offset"] = np.asarray(e.D["cell_offset"]).astype(np.uint32)
    for f in ("Ex", "Ez", "rho"):
        st[f"axis:{f}_m0"] = np.asarray(s.D[f"{f}_m0"][1])
        st[f"axis:{f}_m1"] = np.asarray(s.D[f"{f}_m1"][1])
    return st


def main():
    from oracle.kernels import RefKernels
    K = RefKernels()
    for name, case in CASES.items():
        st = run_case(case, K)
        np.savez_compressed(os.path.join(HERE, name), **st)
        print(name, sum(v.nbytes for v in st.values()) // 1024, "KiB raw")
    for name, case in FULL_RUNS.items():
        st = run_full(case, K)
        np.savez_compressed(os.path.join(HERE, name), **st)
        print(name, sum(np.asarray(v).nbytes for v in st.values()) // 1024, "KiB raw")
    for name in list(BENCH_RUNS) + list(SHAPE_RUNS):
        case, cfg = golden_run(name)
        st = run_full(case, K, cfg=cfg)
        np.savez_compressed(os.path.join(HERE, name), **st)
        print(name, sum(np.asarray(v).nbytes for v in st.values()) // 1024, "KiB raw")


def bench_cfg(case):
    import bench
    cfg = bench.workload(seed=case["seed"])
    if "nppc" in case:
        cfg["eons_in"]["Nppc"] = tuple(case["nppc"])
    return cfg


def main_only(names):
    """Regenerate only the named fixtures."""
    from oracle.kernels import RefKernels
    K = RefKernels()
    for name in names:
        if name in CASES:
            st = run_case(CASES[name], K)
        else:
            case, cfg = golden_run(name)
            st = run_full(case, K, cfg=cfg)
        np.savez_compressed(os.path.join(HERE, name), **st)
        print(name, sum(np.asarray(v).nbytes for v in st.values()) // 1024, "KiB raw")


if __name__ == "__main__":
    import sys
    if len(sys.argv) > 1:
        main_only(sys.argv[1:])
    else:
        main()
