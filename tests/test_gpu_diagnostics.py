"""Records of a real run (FP64 form, diagnostics attached to PIC_loop as the
reference's examples do) against the oracle taken through the reference's
record sequence (diagnostics.py:121-141) at the same iteration; the records
convert to VTK."""
import os

import numpy as np
import pytest

from chimeracl_gb300.diagnostics import Diagnostics, read_record
from chimeracl_gb300.vtk_export import record_to_vtk
from tests.lpa_setup import build_oracle, build_product, small_lpa

pytestmark = pytest.mark.gpu

FIELDS = ["rho", "Ez", "Bx", "By", "Bz"]


def oracle_record(osol, ospecies, fields):
    """diagnostics.py:121-141 on the oracle's objects (sort first, as the
    product does for a record taken before any step)."""
    out = {}
    for fld in fields:
        if fld == "rho" or fld[0] == "J":
            for sp in ospecies:
                sp.sort_parts(grid=osol)
            osol.depose_charge(ospecies)
            osol.fb_transform(scals=[fld], dir=0)
            osol.fields_smooth([fld])
        osol.fb_transform(scals=[fld], dir=1)
        stack = [osol.D[fld + "_m0"][None]]
        for m in range(1, osol.Args["M"] + 1):
            f = osol.D[fld + "_m" + str(m)][None]
            stack += [f.real, f.imag]
        out[fld] = np.concatenate(stack, axis=0)
    return out


def test_records_against_oracle(cuda, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    cfg = small_lpa(Nx=128, Nr=32, M=1, seed=9)
    sol, eons, ions, loop = build_product(cfg, precision="fp64")
    osol, oe, oi, oloop = build_oracle(cfg)
    diag = Diagnostics({"Interval": 10, "ScalarFields": ["rho", "Ez"], "VectorFields": ["B"],
                        "Species": {"Components": ["x", "y", "z", "w", "px"],
                                    "Selections": [("x", -30.0, None)]}},
                       sol, species=[eons], frame=loop.frames[0])
    loop.diags = [diag]
    want = {0: oracle_record(osol, [oe], FIELDS)}
    for _ in range(20):
        oloop.step()
    want[20] = oracle_record(osol, [oe], FIELDS)
    ox = oe.D["x"][:oe.Args["Np"]].copy()
    ow = oe.D["w"][:oe.Args["Np"]].copy()
    for _ in range(21):  # records at 0, 10, 20
        loop.step()
    files = sorted(os.listdir(tmp_path / "diags"))
    assert [f.split(".")[0] for f in files] == ["000000000", "000000010", "000000020"]
    for it in (0, 20):
        rec = read_record(str(tmp_path / "diags" / files[it // 10]))
        assert int(rec["/data/info/iteration"]) == it
        for fld in FIELDS:
            got, ref = rec["/data/fields/" + fld], want[it][fld]
            assert got.dtype == np.float32 and got.shape == ref.shape
            scale = np.abs(ref).max()
            # float32 storage: one rounding of values held to 1e-10 of the oracle
            assert np.abs(got - ref).max() <= 2e-7 * scale, (it, fld)
    rec = read_record(str(tmp_path / "diags" / files[2]))
    base = "/data/species/species_0/"
    sel = ox > -30.0
    np.testing.assert_allclose(rec[base + "x"], ox[sel], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(rec[base + "w"], ow[sel] * eons.Args["w2pC"], rtol=1e-12)
    np.testing.assert_allclose(rec["/data/info/Xgrid"], osol.Args["Xgrid"], rtol=1e-14)
    out = record_to_vtk(str(tmp_path / "diags" / files[2]), str(tmp_path / "vtk"), nt=5)
    assert len(out) == 2 and all(os.path.getsize(p) > 0 for p in out)
