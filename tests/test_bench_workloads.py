"""The benchmark's workload builders, on the CPU: the single run
(2048 x 256, m = 0, 1), the large-mode run (4096 x 512, m = 0..2 with the
astigmatic laser) and the 64 batched small runs (grid sizes, densities and
lasers inside their stated ranges, seeded, the pulse clear of the
absorbing edges)."""
import numpy as np

import bench


def _cells(cfg):
    g = cfg["grid_in"]
    return (g["Xmax"] - g["Xmin"]) / (g["Nx"] - 1), g["Rmax"] / (g["Nr"] - 1.5)


def test_single_and_large_mode_runs():
    c2, c3 = bench.workload(), bench.large_modes_workload()
    assert (c2["grid_in"]["Nx"], c2["grid_in"]["Nr"], c2["grid_in"]["M"]) == (2048, 256, 1)
    assert (c3["grid_in"]["Nx"], c3["grid_in"]["Nr"], c3["grid_in"]["M"]) == (4096, 512, 2)
    assert c3["eons_in"]["Nppc"] == (2, 2, 4) and c3["laser_in"]["astig"] == 0.2
    assert c3["laser_in"]["a0"] == 4.0 and c3["laser_in"]["R"] == 12.0
    # tau = 10 field FWHM: Lx = tau / (2 sqrt(ln 2))
    assert abs(c3["laser_in"]["Lx"] * 2 * np.sqrt(np.log(2)) - 10.0) < 1e-12
    # the large-mode run keeps the single run's cells
    np.testing.assert_allclose(_cells(c3), _cells(c2), rtol=5e-3)
    # (4096 x 512 x 16 macro-electrons ~ 33.5M)
    ne = (c3["grid_in"]["Nx"] - 1) * (c3["grid_in"]["Nr"] - 1) * 16
    assert 33.4e6 < ne < 33.6e6


def test_batched_runs_ranges_and_seeding():
    cases = bench.batched_cases(64, seed=0)
    assert len(cases) == 64
    assert bench.batched_cases(64, seed=0) == cases
    assert bench.batched_cases(64, seed=1) != cases
    for c in cases:
        g, e, las = c["grid_in"], c["eons_in"], c["laser_in"]
        assert g["Nx"] in (256, 384, 512, 768, 1024) and g["Nr"] in (32, 64, 96, 128)
        assert g["M"] == 1 and e["Nppc"] == (1, 1, 4)
        assert 5e-4 <= e["dens"] <= 3e-3 and 1.0 <= las["a0"] <= 3.0 and 4.0 <= las["R"] <= 10.0
        # the pulse (2 Lx either side of x0) lies where the edge damping
        # profile is 1 (beyond 4/3 DampCells cells from either end,
        # solver_methods_cl.py:32-41)
        dx = (g["Xmax"] - g["Xmin"]) / g["Nx"]
        lo = g["Xmin"] + 4.0 / 3.0 * g["DampCells"] * dx
        hi = g["Xmax"] - 4.0 / 3.0 * g["DampCells"] * dx
        assert lo < las["x0"] - 2 * las["Lx"] and las["x0"] + 2 * las["Lx"] < hi
    sizes = {(c["grid_in"]["Nx"], c["grid_in"]["Nr"]) for c in cases}
    assert len(sizes) > 10  # uneven


def test_cpu_oracle_rate_in_a_child_process():
    """The CPU baseline leg (the oracle in a child process without torch,
    OpenMP threads passive): a rate, the thread count and the time come
    back."""
    from tests.lpa_setup import small_lpa
    rate, cores, t = bench.cpu_oracle_rate(small_lpa(Nx=64, Nr=16, M=1), steps=2, warmup=1)
    assert rate > 0 and cores >= 1 and t > 0


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference` (the oracle on the host cores, 1 step):
    one JSON line with the contract's keys, its own rate as e2e, no
    host-device traffic."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True,
                       cwd=root, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e", "steps_timed"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps_timed"] == 1
    assert d["config"]["workload"] == bench.WORKLOAD
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
