"""Legacy VTK output of a zone, in the layout of Typhon's writer.

Typhon writes OUTPUT FORMAT = VTK (ASCII) or VTK-BIN through CFDTOOLS/FileFormat/vtk
(VTKFMT.f90: header; VTKMESH.f90 writevtk_ustmesh: vertices and cells; VTKSOL.f90
writevtk_sol: cell data), called by SOURCE/XIO/output_zone.f90.  This module writes the same
file from a RawMesh (the mesh as read, before preprocessing) and per-cell fields downloaded
from the device:

* header ``# vtk DataFile Version 2.0`` / ``TYPHON`` / ``ASCII`` or ``BINARY``, then
  ``DATASET UNSTRUCTURED_GRID``;
* ``POINTS n double``: every vertex of the mesh, three per line (VTKMESH.f90:61-90);
* ``CELLS ncell ntot``: the cell sections (elements of the mesh's highest dimension) in
  their order, one line per element: its vertex count, then its 0-based vertices
  (VTKMESH.f90:95-124); ``CELL_TYPES``: the VTK type of each (VTKMESH.f90:126-150,
  typhon2vtk_elemtype);
* ``CELL_DATA ncell``, then each scalar (``SCALARS name double`` + ``LOOKUP_TABLE
  default``, one value per line) and each vector (``VECTORS name double``, three per line)
  in the cell order of the sections (VTKSOL.f90:52-199: element i of a section carries the
  value of its cell, the element number).

Numbers are printed as Fortran's ``1P,E17.8E3`` (8 digits after the point, a three-digit
exponent).  The binary form is Typhon's big-endian stream: each header line ends with a
newline, the numbers follow as raw big-endian doubles (vertex indices and types as 32-bit
integers), and a newline closes the vertex, cell-type and field blocks; the cell-type header
of the binary form carries a trailing `` int`` as Typhon writes it.

For a Navier-Stokes zone the fields are Typhon's primitive state (def_model_ns.f90:97-99):
RHO, PS and the vector V; for heat conduction the scalar TS (def_model_kdif.f90:45).
"""
import numpy as np

from .umesh import (DIM, ELEM_BAR2, ELEM_HEXA8, ELEM_PENTA6, ELEM_QUAD4, ELEM_TETRA4, ELEM_TRI3, RawMesh)

VTK_TYPE = {ELEM_BAR2: 3, ELEM_TRI3: 5, ELEM_QUAD4: 9, ELEM_TETRA4: 10, ELEM_PENTA6: 13, ELEM_HEXA8: 12}


def fortran_e(x):
    """x as Fortran's 1P,E17.8E3: d.dddddddd E+xxx, right-justified in 17 characters."""
    x = float(x)
    if x == 0.0:
        s = "0.00000000E+000"
        return (" " * 17 + ("-" + s if np.signbit(x) else s))[-17:]
    m, e = f"{x:.8E}".split("E")
    ex = int(e)
    return f"{m}E{'-' if ex < 0 else '+'}{abs(ex):03d}".rjust(17)


def _cell_sections(raw: RawMesh):
    dmax = max(DIM[t] for t, _, _ in raw.sections)
    out = [(t, np.asarray(ie), np.asarray(cv)) for t, ie, cv in raw.sections if DIM[t] == dmax]
    for t, _, _ in out:
        if t not in VTK_TYPE:
            raise ValueError(f"VTK writer: no VTK type for element type {t}")
    return out


def write_vtk(path, raw: RawMesh, scalars=(), vectors=(), binary=False):
    """Write the mesh and cell fields.  scalars: [(name, values[ncell_int])], vectors:
    [(name, values[3][ncell_int])], both indexed by cell (0-based, element number - 1)."""
    secs = _cell_sections(raw)
    ncell = sum(len(ie) for _, ie, _ in secs)
    ntot = sum((cv.shape[1] + 1) * len(ie) for _, ie, cv in secs)
    cell_order = np.concatenate([ie for _, ie, _ in secs]).astype(np.int64) - 1
    vt = np.asarray(raw.vtex, np.float64)
    with open(path, "wb") as f:
        if binary:
            def line(s):
                f.write(s.encode() + b"\n")

            line("# vtk DataFile Version 2.0")
            line("TYPHON")
            line("BINARY")
            line("DATASET UNSTRUCTURED_GRID")
            line("POINTS %9d double" % len(vt))
            f.write(vt.astype(">f8").tobytes())
            f.write(b"\n")
            line(("CELLS %10d%10d" % (ncell, ntot)).rstrip())
            for _, ie, cv in secs:
                nv = cv.shape[1]
                rec = np.empty((len(ie), nv + 1), ">i4")
                rec[:, 0] = nv
                rec[:, 1:] = cv - 1
                f.write(rec.tobytes())
            line("CELL_TYPES %9d int" % ncell)
            for t, ie, _ in secs:
                f.write(np.full(len(ie), VTK_TYPE[t], ">i4").tobytes())
            f.write(b"\n")
            line("CELL_DATA %9d" % ncell)
            for name, v in scalars:
                line(f"SCALARS {name} double")
                line("LOOKUP_TABLE default")
                f.write(np.asarray(v, np.float64)[cell_order].astype(">f8").tobytes())
                f.write(b"\n")
            for name, v in vectors:
                line(f"VECTORS {name} double")
                f.write(np.asarray(v, np.float64)[:, cell_order].T.astype(">f8").tobytes())
                f.write(b"\n")
            return
        out = ["# vtk DataFile Version 2.0", "TYPHON", "ASCII", "DATASET UNSTRUCTURED_GRID",
               "POINTS %9d double" % len(vt)]
        out += ["".join(fortran_e(x) for x in p) for p in vt]
        out.append("CELLS %10d%10d" % (ncell, ntot))
        for _, ie, cv in secs:
            nv = cv.shape[1]
            out += ["%3d" % nv + "".join("%9d" % (k - 1) for k in row) for row in cv]
        out.append("CELL_TYPES %9d" % ncell)
        for t, ie, _ in secs:
            out += ["%2d" % VTK_TYPE[t]] * len(ie)
        out.append("CELL_DATA %9d" % ncell)
        for name, v in scalars:
            out += [f"SCALARS {name} double", "LOOKUP_TABLE default"]
            out += [fortran_e(x) for x in np.asarray(v, np.float64)[cell_order]]
        for name, v in vectors:
            out.append(f"VECTORS {name} double")
            vv = np.asarray(v, np.float64)[:, cell_order]
            out += ["".join(fortran_e(x) for x in vv[:, i]) for i in range(vv.shape[1])]
        f.write(("\n".join(out) + "\n").encode())


def read_vtk_ascii(path):
    """The sections of an ASCII legacy VTK file written by Typhon or write_vtk: dict of
    'points' (n, 3), 'cells' (list of vertex lists), 'types', and the cell fields by name."""
    lines = open(path).read().split("\n")
    out, i = {}, 4
    while i < len(lines):
        w = lines[i].split()
        if not w:
            i += 1
            continue
        if w[0] == "POINTS":
            n = int(w[1])
            out["points"] = np.array([[float(x) for x in lines[i + 1 + k].split()] for k in range(n)])
            i += 1 + n
        elif w[0] == "CELLS":
            n = int(w[1])
            out["cells"] = [[int(x) for x in lines[i + 1 + k].split()[1:]] for k in range(n)]
            i += 1 + n
        elif w[0] == "CELL_TYPES":
            n = int(w[1])
            out["types"] = [int(lines[i + 1 + k]) for k in range(n)]
            i += 1 + n
        elif w[0] == "CELL_DATA":
            out["ncell"] = int(w[1])
            i += 1
        elif w[0] == "SCALARS":
            n = out["ncell"]
            out[w[1]] = np.array([float(lines[i + 2 + k]) for k in range(n)])
            i += 2 + n
        elif w[0] == "VECTORS":
            n = out["ncell"]
            out[w[1]] = np.array([[float(x) for x in lines[i + 1 + k].split()] for k in range(n)]).T
            i += 1 + n
        else:
            raise ValueError(f"{path}: unexpected line {lines[i]!r}")
    return out
