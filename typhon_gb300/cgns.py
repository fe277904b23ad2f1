"""CGNS unstructured meshes stored in the ADF format, read without libcgns.

Typhon reads CGNS meshes through libcgns (CFDTOOLS/FileFormat/cgns/readcgnszone.f90,
readcgnsvtex.f90, readcgns_ustconnect.f90, readcgns_ustboco.f90).  This module reads the
same files directly: the ADF container (a tree of nodes, each with a name, a label, a data
type, dimensions and one data chunk) and, inside it, the CGNS layout of an unstructured zone.
The result is a ``RawMesh`` (nodes, element sections, boundary marks) that ``preprocess``
turns into a mesh description exactly as it does for a .tym file.

What Typhon takes from the file, and how it is mapped:

* coordinates ``GridCoordinates/CoordinateX|Y|Z`` (doubles; a missing Z is 0);
* ``Elements_t`` sections in file order: NODE sections are skipped; linear elements keep
  their element numbers (``ElementRange``); MIXED sections are split per element type in
  increasing CGNS type code, element numbers kept (readcgns_ustconnect.f90:118-152);
  quadratic and NGON elements are refused;
* ``ZoneBC/BC_t`` in file order: the family is the ``FamilyName`` child, else the BC's
  name; tags are ``PointList`` (``ElementList`` counts as face elements); the location is
  the ``GridLocation`` child (FaceCenter: face element numbers, Vertex: vertex numbers;
  missing: Vertex, as Typhon assumes); ``PointRange`` and family-specified BCs are refused,
  as in readcgns_ustboco.f90:47-104.

ADF layout (as stored by the ADF core of the CGNS library): ASCII hex "disk pointers" of
12 characters (8 for a 4096-byte block number, 4 for the offset in the block); a file header
whose ``AdF2`` field gives the byte order of the binary data (``B`` big, ``L`` little
endian) and whose ``AdF4`` field starts with the root node's pointer; node records
``NoDe`` name(32) label(32) nsub(8 hex) nentries(8 hex) sub-node-table pointer(12)
type(32) ndim(2 hex) dims(12 x 8 hex) nchunks(4 hex) data pointer(12) ``TaiL``; sub-node
tables ``SNTb`` end pointer(12) then entries name(32) pointer(12), unused entries named
"unused entry in sub-node-table"; data chunks ``DaTa`` end pointer(12) data ``dEnD``.
"""
from dataclasses import dataclass

import numpy as np

from .umesh import ELEM_BAR2, ELEM_HEXA8, ELEM_PENTA6, ELEM_QUAD4, ELEM_TETRA4, ELEM_TRI3, RawMesh

_NODE_BYTES = 246
_UNUSED = "unused entry in sub-node-table"
_TYPE_SIZE = {"I4": 4, "I8": 8, "U4": 4, "U8": 8, "R4": 4, "R8": 8, "C1": 1, "B1": 1}
_TYPE_NUMPY = {"I4": "i4", "I8": "i8", "U4": "u4", "U8": "u8", "R4": "f4", "R8": "f8", "B1": "u1"}

# CGNS ElementType_t codes -> Typhon element types, with vertices per element
CGNS_NODE, CGNS_MIXED = 2, 20
_CGNS_LINEAR = {3: (ELEM_BAR2, 2), 5: (ELEM_TRI3, 3), 7: (ELEM_QUAD4, 4), 10: (ELEM_TETRA4, 4),
                14: (ELEM_PENTA6, 6), 17: (ELEM_HEXA8, 8)}
_CGNS_PYRA5 = 12


class CgnsError(ValueError):
    pass


@dataclass
class AdfNode:
    name: str
    label: str
    dtype: str
    dims: tuple
    nsub: int
    nentries: int
    table: int      # byte offset of the sub-node table
    nchunks: int
    data_at: int    # byte offset of the data chunk


class AdfFile:
    """Read-only view of an ADF file held in memory."""

    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        # the "@(#)" prefix is sometimes stored with the high bit set: test the rest
        if self.b[4:16] != b"ADF Database":
            raise CgnsError(f"{path}: not an ADF file")
        i = self.b.find(b"AdF2", 0, 256)
        j = self.b.find(b"AdF4", 0, 256)
        if i < 0 or j < 0:
            raise CgnsError(f"{path}: ADF header fields missing")
        fmt = chr(self.b[i + 4])
        if fmt not in "BL":
            raise CgnsError(f"{path}: unsupported ADF number format {fmt!r}")
        self.endian = ">" if fmt == "B" else "<"
        self.root = self.node(self._ptr(j + 4))

    def _hex(self, at, n):
        return int(self.b[at:at + n], 16)

    def _ptr(self, at):
        return self._hex(at, 8) * 4096 + self._hex(at + 8, 4)

    def _str(self, at, n):
        return self.b[at:at + n].decode("ascii", "replace").rstrip(" \x00")

    def node(self, at):
        if self.b[at:at + 4] != b"NoDe" or self.b[at + _NODE_BYTES - 4:at + _NODE_BYTES] != b"TaiL":
            raise CgnsError(f"no ADF node at byte {at}")
        q = at + 4
        name, label = self._str(q, 32), self._str(q + 32, 32)
        nsub, nent, table = self._hex(q + 64, 8), self._hex(q + 72, 8), self._ptr(q + 80)
        dtype = self._str(q + 92, 32)
        ndim = self._hex(q + 124, 2)
        dims = tuple(self._hex(q + 126 + 8 * k, 8) for k in range(ndim))
        nch, data_at = self._hex(q + 222, 4), self._ptr(q + 226)
        return AdfNode(name, label, dtype, dims, nsub, nent, table, nch, data_at)

    def children(self, n):
        if n.nsub == 0:
            return []
        if self.b[n.table:n.table + 4] != b"SNTb":
            raise CgnsError(f"node {n.name}: no sub-node table")
        out, q = [], n.table + 16
        for _ in range(n.nentries):
            nm = self._str(q, 32)
            if nm != _UNUSED:
                out.append(self.node(self._ptr(q + 32)))
            q += 44
        if len(out) != n.nsub:
            raise CgnsError(f"node {n.name}: {len(out)} children listed, {n.nsub} expected")
        return out

    def child(self, n, name=None, label=None):
        for c in self.children(n):
            if (name is None or c.name == name) and (label is None or c.label == label):
                return c
        return None

    def data(self, n):
        """The node's data: a numpy array shaped as the node's dimensions (first index
        fastest, as in Fortran), a string for C1 data, or None for a node without data."""
        if n.dtype == "MT" or n.nchunks == 0:
            return None
        if n.nchunks != 1:
            raise CgnsError(f"node {n.name}: data in {n.nchunks} chunks is not supported")
        if n.dtype not in _TYPE_SIZE:
            raise CgnsError(f"node {n.name}: data type {n.dtype} is not supported")
        at = n.data_at
        if self.b[at:at + 4] != b"DaTa":
            raise CgnsError(f"node {n.name}: no data chunk")
        count = int(np.prod(n.dims)) if n.dims else 1
        raw = self.b[at + 16:at + 16 + count * _TYPE_SIZE[n.dtype]]
        if n.dtype == "C1":
            return raw.decode("ascii", "replace").rstrip(" \x00")
        a = np.frombuffer(raw, self.endian + _TYPE_NUMPY[n.dtype]).astype(_TYPE_NUMPY[n.dtype])
        return a.reshape(n.dims[::-1]).T if len(n.dims) > 1 else a


def read_cgns(path, base=1, zone=1) -> RawMesh:
    """The unstructured zone `zone` of base `base` (1-based, Typhon's defaults) as a RawMesh."""
    f = AdfFile(path)
    bases = [c for c in f.children(f.root) if c.label == "CGNSBase_t"]
    if not 1 <= base <= len(bases):
        raise CgnsError(f"{path}: no base {base}")
    zones = [c for c in f.children(bases[base - 1]) if c.label == "Zone_t"]
    if not 1 <= zone <= len(zones):
        raise CgnsError(f"{path}: no zone {zone}")
    z = zones[zone - 1]
    zt = f.child(z, label="ZoneType_t")
    if zt is None or f.data(zt) != "Unstructured":
        raise CgnsError("only unstructured CGNS zones are supported")
    nvtex = int(np.asarray(f.data(z)).reshape(-1)[0])

    gc = f.child(z, label="GridCoordinates_t")
    if gc is None:
        raise CgnsError("zone without GridCoordinates")
    xyz = np.zeros((nvtex, 3))
    for k, nm in enumerate(("CoordinateX", "CoordinateY", "CoordinateZ")):
        c = f.child(gc, name=nm)
        if c is None:
            if k < 2:
                raise CgnsError(f"missing {nm}")
            continue
        xyz[:, k] = np.asarray(f.data(c), np.float64)[:nvtex]

    raw = RawMesh(vtex=xyz)
    for sec in (c for c in f.children(z) if c.label == "Elements_t"):
        etype = int(np.asarray(f.data(sec)).reshape(-1)[0])
        er = f.child(sec, name="ElementRange")
        ec = f.child(sec, name="ElementConnectivity")
        if er is None or ec is None:
            raise CgnsError(f"section {sec.name}: ElementRange or ElementConnectivity missing")
        ista, iend = (int(v) for v in np.asarray(f.data(er)).reshape(-1)[:2])
        conn = np.asarray(f.data(ec), np.int32).reshape(-1)
        nelem = iend - ista + 1
        if etype == CGNS_NODE:
            continue
        if etype in _CGNS_LINEAR:
            typ, nv = _CGNS_LINEAR[etype]
            raw.sections.append((typ, np.arange(ista, iend + 1, dtype=np.int32),
                                 conn[:nelem * nv].reshape(nelem, nv).copy()))
        elif etype == CGNS_MIXED:
            # element k: type code then its vertices (sort_elementtype, readcgns_ustconnect.f90:180-210)
            types, starts, pos = [], [], 0
            while pos < conn.size:
                t = int(conn[pos])
                if t not in _CGNS_LINEAR:
                    raise CgnsError(f"section {sec.name}: element type {t} in a MIXED section is not supported")
                types.append(t)
                starts.append(pos + 1)
                pos += 1 + _CGNS_LINEAR[t][1]
            if len(types) != nelem or pos != conn.size:
                raise CgnsError(f"section {sec.name}: unexpected end of MIXED section")
            types, starts = np.array(types), np.array(starts)
            for t in sorted(set(types.tolist())):
                sel = np.nonzero(types == t)[0]
                typ, nv = _CGNS_LINEAR[t]
                cv = np.stack([conn[s:s + nv] for s in starts[sel]]).astype(np.int32)
                raw.sections.append((typ, (ista + sel).astype(np.int32), cv))
        elif etype == _CGNS_PYRA5:
            raise CgnsError("PYRA_5 elements are not supported by the mesh preprocessing")
        else:
            raise CgnsError(f"section {sec.name}: CGNS element type {etype} is not supported")
    if not raw.sections:
        raise CgnsError("zone without elements")

    zbc = f.child(z, label="ZoneBC_t")
    for bc in (f.children(zbc) if zbc is not None else []):
        if bc.label != "BC_t":
            continue
        if f.data(bc) == "FamilySpecified":
            raise CgnsError(f"BC {bc.name}: family-specified boundary conditions are not supported")
        fam = f.child(bc, label="FamilyName_t")
        family = f.data(fam) if fam is not None else bc.name
        loc = f.child(bc, label="GridLocation_t")
        where = f.data(loc) if loc is not None else "Vertex"
        pl = f.child(bc, name="PointList")
        el = f.child(bc, name="ElementList")
        if pl is None and el is None:
            raise CgnsError(f"BC {bc.name}: only PointList or ElementList tags are supported")
        tags = np.asarray(f.data(pl if pl is not None else el), np.int32).reshape(-1)
        if el is not None and pl is None:
            where = "FaceCenter"
        if where == "Vertex":
            raw.marks.append((family, tags, "vertex"))
        elif where == "FaceCenter":
            raw.marks.append((family, tags))
        else:
            raise CgnsError(f"BC {bc.name}: grid location {where} is not supported")
    return raw
