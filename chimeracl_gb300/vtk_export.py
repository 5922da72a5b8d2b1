"""Records -> VTK files, headless (the reference's chimera2VTK.py, without
its tvtk, numba, h5py and mpi4py dependencies).

Fields become a structured grid (``fields_<it>.vts``) of Nt azimuthal planes
x Nr radii x Nx positions -- the point order of chimera2VTK.py:48-63: angle
fastest, then radius, then x -- carrying each recorded field rebuilt from its
modes as F_0 + sum_m 2 Re(F_m e^{i m theta}) (chimera2VTK.py:66-85), with the
reference's axis treatment (row 0 of mode 0 copied from row 1, of modes >= 1
set to zero) and the ghost radius clamped to 0.  Species become point sets
(``species_<i>_<it>.vtp``) carrying every recorded component but x, y, z.  In
a moving frame x is shifted by iteration * dt * FrameVelocity.

The files are VTK XML with the arrays in one raw appended block (Float32,
little endian, a UInt64 byte count before each array), which ParaView and
the VTK readers open directly.

Usage: ``python -m chimeracl_gb300.vtk_export diags/ [latest] [--nt 25]
[--out vtk]``."""
import argparse
import os
import sys

import numpy as np

from .diagnostics import read_record


def _xml_file(kind, body, blobs, path):
    """Write a VTK XML file whose DataArrays (in `body`, with offsets in
    order) read the raw blocks `blobs`."""
    with open(path, "wb") as f:
        f.write(('<?xml version="1.0"?>\n<VTKFile type="%s" version="1.0" '
                 'byte_order="LittleEndian" header_type="UInt64">\n' % kind).encode())
        f.write(body.encode())
        f.write(b'  <AppendedData encoding="raw">\n   _')
        for b in blobs:
            f.write(np.uint64(len(b)).tobytes())
            f.write(b)
        f.write(b"\n  </AppendedData>\n</VTKFile>\n")


def _arrays(named, offset=0):
    """DataArray tags and raw blocks for [(name, float32 array, ncomp)]."""
    tags, blobs = [], []
    for name, a, nc in named:
        b = np.ascontiguousarray(a, dtype="<f4").tobytes()
        nattr = ' NumberOfComponents="%d"' % nc if nc > 1 else ""
        nm = ' Name="%s"' % name if name else ""
        tags.append('<DataArray type="Float32"%s%s format="appended" offset="%d"/>'
                    % (nm, nattr, offset))
        blobs.append(b)
        offset += 8 + len(b)
    return tags, blobs, offset


def field_planes(data, theta):
    """A recorded field, shape (1 + 2M, Nr, Nx), on the planes `theta`:
    array (Nx, Nr, Nt) of F_0 + sum_m 2 Re(F_m e^{i m theta})."""
    data = np.array(data, dtype=np.float64)
    m0 = data[0].copy()
    m0[0] = m0[1]  # axis treatment (chimera2VTK.py:130-131)
    out = np.repeat(m0.T[:, :, None], theta.size, axis=2)
    for k, m in enumerate(range(1, (data.shape[0] - 1) // 2 + 1)):
        fm = data[1 + 2 * k] + 1j * data[2 + 2 * k]
        fm[0] = 0  # axis treatment (chimera2VTK.py:135-137)
        out += 2 * np.real(fm.T[:, :, None] * np.exp(1j * m * theta)[None, None, :])
    return out


def grid_points(xgrid, rgrid, theta):
    """Points (Nx, Nr, Nt, 3): (x, r cos theta, r sin theta)."""
    X = np.broadcast_to(xgrid[:, None, None], (xgrid.size, rgrid.size, theta.size))
    Y = rgrid[None, :, None] * np.cos(theta)[None, None, :]
    Z = rgrid[None, :, None] * np.sin(theta)[None, None, :]
    return np.stack([X, np.broadcast_to(Y, X.shape), np.broadcast_to(Z, X.shape)], axis=-1)


def record_to_vtk(fname, out_dir="vtk", nt=25):
    """Convert one record; returns the files written."""
    rec = read_record(fname)
    it = int(os.path.basename(fname).split(".")[0])
    info = "/data/info/"
    dt, vel = float(rec[info + "dt"]), float(rec[info + "FrameVelocity"])
    x0 = it * dt * vel
    xgrid = np.asarray(rec[info + "Xgrid"], dtype=np.float64) - x0
    rgrid = np.asarray(rec[info + "Rgrid"], dtype=np.float64)
    rgrid = rgrid * (rgrid > 0)
    theta = 2 * np.pi / (nt - 1) * np.arange(nt)
    os.makedirs(out_dir, exist_ok=True)
    written = []
    fields = sorted(k for k in rec if k.startswith("/data/fields/"))
    if fields:
        nx, nr = xgrid.size, rgrid.size
        named = [(k.rsplit("/", 1)[1], field_planes(rec[k], theta), 1) for k in fields]
        tags, blobs, off = _arrays(named)
        ptag, pblob, _ = _arrays([("", grid_points(xgrid, rgrid, theta), 3)], off)
        ext = "0 %d 0 %d 0 %d" % (nt - 1, nr - 1, nx - 1)
        body = ('  <StructuredGrid WholeExtent="%s">\n   <Piece Extent="%s">\n'
                '    <PointData>\n     %s\n    </PointData>\n'
                '    <Points>\n     %s\n    </Points>\n   </Piece>\n  </StructuredGrid>\n'
                % (ext, ext, "\n     ".join(tags), ptag[0]))
        path = os.path.join(out_dir, "fields_%d.vts" % it)
        _xml_file("StructuredGrid", body, blobs + pblob, path)
        written.append(path)
    species = sorted({k.split("/")[3] for k in rec if k.startswith("/data/species/")})
    for sp in species:
        base = "/data/species/" + sp + "/"
        n = np.asarray(rec[base + "x"]).size
        pts = np.stack([np.asarray(rec[base + "x"]) - x0, np.asarray(rec[base + "y"]),
                        np.asarray(rec[base + "z"])], axis=-1)
        comps = sorted(k[len(base):] for k in rec if k.startswith(base)
                       and k[len(base):] not in ("x", "y", "z"))
        tags, blobs, off = _arrays([(c, rec[base + c], 1) for c in comps])
        ptag, pblob, off = _arrays([("", pts, 3)], off)
        # one vertex cell per particle, so that viewers draw them as points
        conn = np.arange(n, dtype="<i8").tobytes()
        offs = np.arange(1, n + 1, dtype="<i8").tobytes()
        vtag = ('<DataArray type="Int64" Name="connectivity" format="appended" offset="%d"/>'
                '<DataArray type="Int64" Name="offsets" format="appended" offset="%d"/>'
                % (off, off + 8 + len(conn)))
        body = ('  <PolyData>\n   <Piece NumberOfPoints="%d" NumberOfVerts="%d" '
                'NumberOfLines="0" NumberOfStrips="0" NumberOfPolys="0">\n'
                '    <PointData>\n     %s\n    </PointData>\n    <Points>\n     %s\n'
                '    </Points>\n    <Verts>%s</Verts>\n   </Piece>\n  </PolyData>\n'
                % (n, n, "\n     ".join(tags), ptag[0], vtag))
        path = os.path.join(out_dir, "%s_%d.vtp" % (sp, it))
        _xml_file("PolyData", body, blobs + pblob + [conn, offs], path)
        written.append(path)
    return written


def main(argv=None):
    ap = argparse.ArgumentParser(description="chimeracl_gb300 records -> VTK")
    ap.add_argument("path")
    ap.add_argument("selection", nargs="?", default=None, help="'latest': last record only")
    ap.add_argument("--nt", type=int, default=25, help="azimuthal planes")
    ap.add_argument("--out", default="vtk")
    args = ap.parse_args(argv)
    recs = sorted(f for f in os.listdir(args.path) if f.endswith((".h5", ".npz")))
    if args.selection == "latest":
        recs = recs[-1:]
    for r in recs:
        record_to_vtk(os.path.join(args.path, r), args.out, args.nt)
        print("done " + r)
    return 0


if __name__ == "__main__":
    sys.exit(main())
