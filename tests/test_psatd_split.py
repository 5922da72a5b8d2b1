"""The cancellation-free form of the PSATD update (ccl_psatd_advance_split,
the FP32 form's field push) on the CPU: in float64 it equals the reference's
advance_e_g_m (the oracle, solver_ms_pic.cl:57-143) to rounding; evaluated in
float32 it keeps the charge and current response of long-wavelength modes
(w dt ~ 1e-3) to ~1e-6, where the reference's grouping of the same update
keeps one or two digits."""
import numpy as np
import pytest

from chimeracl_gb300.methods.solver_methods_cu import psatd_split_coefficients

DT = 0.039


def _modes(n, rng, xmin=1e-3, xmax=3.0):
    # w dt spread log-uniformly over [xmin, xmax]: long waves to the grid's top
    return np.exp(rng.uniform(np.log(xmin), np.log(xmax), n)) / DT


def _fields(n, rng, dtype=np.complex128, sources_only=False):
    f = [(rng.normal(size=n) + 1j * rng.normal(size=n)).astype(dtype) for _ in range(15)]
    if sources_only:  # E = G = 0: the update is the response to J, dN0, dN1 alone
        for k in range(6):
            f[k][:] = 0
    return f


def split_update(coef, f):
    """numpy evaluation of ccl_psatd_advance_split's arithmetic, in the
    arrays' own precision."""
    c = [coef[..., k] for k in range(8)]
    c1, c2, s, s2, q2, a2, b2, d2 = c
    out = [a.copy() for a in f]
    for k in range(3):
        e0, g0, j0, n0, n1 = f[k], f[3 + k], f[6 + k], f[9 + k], f[12 + k]
        out[k] = c1 * e0 + s * g0 - s2 * j0 + a2 * n0 + b2 * n1
        out[3 + k] = -c2 * e0 + c1 * g0 + q2 * j0 + d2 * (n0 - n1) - s2 * n0
    return out


def reference_update(w, dt, f, real):
    """The reference's expression order (solver_ms_pic.cl:118-126) with its
    coefficients rounded to `real` (what an FP32 port of it computes)."""
    c1 = np.cos(w * dt).astype(real)
    c2 = (np.sin(w * dt) * w).astype(real)
    c3 = (1.0 / w ** 2).astype(real)
    dti, pi2, one = real(1.0 / dt), real(2 * np.pi), real(1)
    out = [a.copy() for a in f]
    for k in range(3):
        e0, g0 = f[k], f[3 + k]
        j0, n0, n1 = f[6 + k] * pi2, f[9 + k] * pi2, f[12 + k] * pi2
        out[k] = c1 * e0 + c2 * c3 * (g0 - j0) + c3 * (c1 * n0 - n1 - (n0 - n1) * dti * c2 * c3)
        out[3 + k] = -c2 * e0 + c1 * (g0 - j0) + j0 + c3 * (dti * (one - c1) * (n0 - n1) - c2 * n0)
    return out


def test_split_equals_reference_in_float64(port):
    rng = np.random.default_rng(0)
    w = _modes(4096, rng)
    f = _fields(w.size, rng)
    ref = [a.copy() for a in f]
    port.advance_e_g_m(1.0 / DT, np.cos(w * DT), np.sin(w * DT) * w, 1.0 / w ** 2, ref)
    got = split_update(psatd_split_coefficients(w, DT), f)
    # the bound is the reference grouping's own float64 cancellation at
    # w dt = 1e-3 (16 digits less log10(1/x^2) = 6)
    for k in range(6):
        scale = np.abs(ref[k]).max()
        assert np.abs(got[k] - ref[k]).max() <= 1e-10 * scale, k


@pytest.mark.parametrize("x", [1e-3, 3e-3, 1e-2, 0.05, 0.0999, 0.1001, 0.3, 1.0, 2.5])
def test_coefficients_against_50_digit_evaluation(x):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50
    w = x / DT
    coef = psatd_split_coefficients(np.array([w]), DT)[0]
    X, W, D, P2 = mp.mpf(x), mp.mpf(x) / mp.mpf(DT), mp.mpf(DT), 2 * mp.pi
    want = [mp.cos(X), W * mp.sin(X), mp.sin(X) / W, P2 * mp.sin(X) / W, P2 * (1 - mp.cos(X)),
            P2 * (mp.cos(X) - mp.sin(X) / X) / W ** 2, P2 * (mp.sin(X) / X - 1) / W ** 2,
            P2 * (1 - mp.cos(X)) / (W ** 2 * D)]
    # (stored in FP32: 1e-13 is far inside what they need; the direct forms
    # just above x = 0.1 lose two digits of float64)
    for k in range(8):
        assert abs(coef[k] - float(want[k])) <= 1e-13 * abs(float(want[k])), (k, coef[k], want[k])


def test_split_keeps_long_wave_sources_in_float32(port):
    rng = np.random.default_rng(1)
    w = _modes(4096, rng, xmin=1e-3, xmax=1e-2)
    f64 = _fields(w.size, rng, sources_only=True)
    exact = [a.copy() for a in f64]
    port.advance_e_g_m(1.0 / DT, np.cos(w * DT), np.sin(w * DT) * w, 1.0 / w ** 2, exact)
    f32 = [a.astype(np.complex64) for a in f64]
    split = split_update(psatd_split_coefficients(w, DT).astype(np.float32), f32)
    refm = reference_update(w, DT, f32, np.float32)
    for k in range(6):
        scale = np.linalg.norm(exact[k])
        e_split = np.linalg.norm(split[k] - exact[k]) / scale
        e_ref = np.linalg.norm(refm[k] - exact[k]) / scale
        assert e_split < 1e-6, (k, e_split)
        assert e_ref > 100 * e_split, (k, e_ref, e_split)
