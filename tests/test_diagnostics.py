"""Records and their VTK export on the CPU: the reference's layout and
quirks (diagnostics.py) with stub solver and species objects, and the VTK
files read back and compared with chimera2VTK.py's reconstruction."""
import os
import re

import numpy as np
import pytest
import torch

from chimeracl_gb300.diagnostics import Diagnostics, read_record
from chimeracl_gb300.vtk_export import field_planes, record_to_vtk


class _Args(dict):
    pass


class StubSolver:
    """Args and DataDev of a 2-mode grid; the transforms only log calls."""

    def __init__(self, rng, Nr=5, Nx=7, M=1):
        self.Args = _Args(Xgrid=np.linspace(-3, 0, Nx), Rgrid=(np.arange(Nr) - 0.5) * 0.4,
                          dx=0.5, dr=0.4, dt=0.49, Nx=Nx, Nr=Nr, M=M)
        self.DataDev = {}
        for f in ("rho", "Ez", "Bx", "By", "Bz"):
            self.DataDev[f + "_m0"] = torch.from_numpy(rng.normal(size=(Nr, Nx)))
            for m in range(1, M + 1):
                self.DataDev[f + "_m" + str(m)] = torch.from_numpy(
                    rng.normal(size=(Nr, Nx)) + 1j * rng.normal(size=(Nr, Nx)))
        self.log = []

    def depose_charge(self, species):
        self.log.append(("depose", len(species)))

    def fb_transform(self, scals=(), vects=(), dir=0):
        self.log.append(("fb", tuple(scals), dir))

    def fields_smooth(self, flds):
        self.log.append(("smooth", tuple(flds)))


class StubSpecies:
    def __init__(self, rng, n=50):
        self.Args = {"Np": n, "w2pC": 3.5}
        self.DataDev = {k: torch.from_numpy(rng.normal(size=n + 3)) for k in
                        ("x", "y", "z", "px", "w")}  # arrays longer than Np
        self.sorted = 0

    def sort_parts(self, grid):
        self.sorted += 1


class StubFrame:
    Args = {"Velocity": 1.0}


@pytest.fixture
def cwd(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    return tmp_path


def test_record_layout_and_quirks(cwd):
    rng = np.random.default_rng(0)
    sol, sp = StubSolver(rng), StubSpecies(rng)
    cfg = {"Interval": 5, "ScalarFields": ["rho", "Ez"], "VectorFields": ["B"],
           "Species": {"Components": ["x", "w", "px"], "Selections": [("x", -0.5, None)]}}
    os.makedirs(cwd / "diags")
    (cwd / "diags" / "stale.txt").write_text("old")
    d = Diagnostics(cfg, sol, species=[sp], frame=StubFrame())
    assert os.listdir(cwd / "diags") == []  # an existing directory is emptied
    d.make_record(3)  # not a multiple of Interval: nothing
    assert os.listdir(cwd / "diags") == []
    d.make_record(10)
    files = os.listdir(cwd / "diags")
    assert len(files) == 1 and re.fullmatch(r"000000010\.(h5|npz)", files[0])
    rec = read_record(str(cwd / "diags" / files[0]))
    info = "/data/info/"
    assert int(rec[info + "iteration"]) == 10 and float(rec[info + "FrameVelocity"]) == 1.0
    for k in ("dx", "dr", "dt", "Nx", "Nr", "M"):
        assert float(rec[info + k]) == float(sol.Args[k])
    np.testing.assert_array_equal(rec[info + "Xgrid"], sol.Args["Xgrid"])
    # fields: [m0, Re m1, Im m1] in float32
    for f in ("rho", "Ez", "Bx", "By", "Bz"):
        a = rec["/data/fields/" + f]
        assert a.dtype == np.float32 and a.shape == (3, 5, 7)
        np.testing.assert_array_equal(a[0], sol.DataDev[f + "_m0"].numpy().astype(np.float32))
        m1 = sol.DataDev[f + "_m1"].numpy()
        np.testing.assert_array_equal(a[1], m1.real.astype(np.float32))
        np.testing.assert_array_equal(a[2], m1.imag.astype(np.float32))
    # rho: deposit, forward, smooth, backward (diagnostics.py:126-131);
    # Ez and B only backward
    assert sol.log[:4] == [("depose", 1), ("fb", ("rho",), 0), ("smooth", ("rho",)),
                           ("fb", ("rho",), 1)]
    assert sol.log[4:] == [("fb", (f,), 1) for f in ("Ez", "Bx", "By", "Bz")]
    assert sp.sorted == 1
    # species: first Np entries, selection x > -0.5, w scaled by w2pC
    x = sp.DataDev["x"].numpy()[:50]
    sel = x > -0.5
    base = "/data/species/species_0/"
    np.testing.assert_array_equal(rec[base + "x"], x[sel])
    np.testing.assert_array_equal(rec[base + "px"], sp.DataDev["px"].numpy()[:50][sel])
    np.testing.assert_allclose(rec[base + "w"], sp.DataDev["w"].numpy()[:50][sel] * 3.5,
                               rtol=1e-15)
    assert rec[base + "x"].dtype == np.float64


def test_empty_species_and_config_w2pC(cwd):
    rng = np.random.default_rng(1)
    sol, sp = StubSolver(rng), StubSpecies(rng)
    sp.Args["Np"] = 0
    d = Diagnostics({"Interval": 1, "Species": {"Components": ["x", "w"]}, "w2pC": 2.0},
                    sol, species=[sp], path="out")
    d.make_record(0)
    f = os.listdir(cwd / "out")[0]
    rec = read_record(str(cwd / "out" / f))
    assert rec["/data/species/species_0/x"].size == 0
    assert not any(k.startswith("/data/fields/") for k in rec)
    assert float(rec["/data/info/FrameVelocity"]) == 0.0


def _read_vtk(path):
    """The XML header and the raw appended arrays of a written VTK file."""
    raw = open(path, "rb").read()
    head, _, tail = raw.partition(b'<AppendedData encoding="raw">\n   _')
    head = head.decode()
    arrays = {}
    for m in re.finditer(r'<DataArray type="(\w+)"(?: Name="(\w*)")?(?: NumberOfComponents="(\d)")?'
                         r' format="appended" offset="(\d+)"/>', head):
        typ, name, nc, off = m.group(1), m.group(2) or "Points", m.group(3), int(m.group(4))
        n = int(np.frombuffer(tail[off:off + 8], "<u8")[0])
        dt = {"Float32": "<f4", "Int64": "<i8"}[typ]
        a = np.frombuffer(tail[off + 8:off + 8 + n], dt)
        arrays[name] = a.reshape(-1, int(nc)) if nc else a
    return head, arrays


def test_vtk_export_matches_chimera2vtk_reconstruction(cwd):
    rng = np.random.default_rng(2)
    Nr, Nx, it, dt, nt = 6, 9, 40, 0.1, 7
    xg, rg = np.linspace(-5, 3, Nx), (np.arange(Nr) - 0.5) * 0.3
    fld = rng.normal(size=(5, Nr, Nx)).astype(np.float32)  # M = 2
    rec = {"data/info/dt": np.asarray(dt), "data/info/FrameVelocity": np.asarray(1.0),
           "data/info/Xgrid": xg, "data/info/Rgrid": rg, "data/fields/Ez": fld,
           "data/species/species_0/x": rng.normal(size=11),
           "data/species/species_0/y": rng.normal(size=11),
           "data/species/species_0/z": rng.normal(size=11),
           "data/species/species_0/w": rng.normal(size=11)}
    os.makedirs(cwd / "d")
    np.savez(cwd / "d" / ("%09d.npz" % it), **rec)
    out = record_to_vtk(str(cwd / "d" / ("%09d.npz" % it)), str(cwd / "vtk"), nt=nt)
    assert sorted(os.path.basename(p) for p in out) == ["fields_40.vts", "species_0_40.vtp"]
    head, arr = _read_vtk(str(cwd / "vtk" / "fields_40.vts"))
    assert 'WholeExtent="0 %d 0 %d 0 %d"' % (nt - 1, Nr - 1, Nx - 1) in head
    theta = 2 * np.pi / (nt - 1) * np.arange(nt)
    x0 = it * dt
    pts = arr["Points"].reshape(Nx, Nr, nt, 3)
    r = rg * (rg > 0)
    np.testing.assert_allclose(pts[..., 0], np.broadcast_to((xg - x0)[:, None, None], (Nx, Nr, nt)),
                               rtol=1e-6)
    shape = (Nx, Nr, nt)
    np.testing.assert_allclose(pts[..., 1], np.broadcast_to(r[None, :, None] * np.cos(theta), shape),
                               atol=1e-6)
    np.testing.assert_allclose(pts[..., 2], np.broadcast_to(r[None, :, None] * np.sin(theta), shape),
                               atol=1e-6)
    # chimera2VTK.py:66-85 and 127-140, written out point by point
    ez = arr["Ez"].reshape(Nx, Nr, nt)
    f = fld.astype(np.float64)
    for ix in (0, 4, Nx - 1):
        for ir in (0, 1, Nr - 1):
            for k in (0, 3):
                v = f[0, max(ir, 1), ix]
                for m in (1, 2):
                    c = (f[2 * m - 1, ir, ix] + 1j * f[2 * m, ir, ix]) if ir > 0 else 0
                    v += 2 * np.real(c * np.exp(1j * m * theta[k]))
                assert abs(ez[ix, ir, k] - v) <= 1e-5 * (1 + abs(v))
    np.testing.assert_allclose(field_planes(fld, theta), ez, rtol=1e-6, atol=1e-6)
    head, arr = _read_vtk(str(cwd / "vtk" / "species_0_40.vtp"))
    assert 'NumberOfPoints="11"' in head
    np.testing.assert_allclose(arr["Points"][:, 0], rec["data/species/species_0/x"] - x0, rtol=1e-6)
    np.testing.assert_allclose(arr["w"], rec["data/species/species_0/w"], rtol=1e-6)
    np.testing.assert_array_equal(arr["connectivity"], np.arange(11))
    np.testing.assert_array_equal(arr["offsets"], np.arange(1, 12))
