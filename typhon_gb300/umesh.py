"""Element meshes: Typhon's .tym (XBIN) format, synthetic generators, and preprocessing.

``RawMesh`` holds what a .tym file holds (nodes, element sections, boundary marks).
``preprocess`` runs the library's native preprocessing (ty_umesh_*, the equivalent of
Typhon's grid_preproc + init_connect_grid) and returns a ``MeshDesc`` with the arrays that
``ty_mesh_create`` takes.

Formats and conventions restated from the reference:
  XBIN stream header and data sections   CFDTOOLS/FileFormat/internal/XBIN_IO.f90:70-135,
                                         XBIN_DATA.f90:139-215
  TYPHON mesh sections                   CFDTOOLS/FileFormat/internal/TYFMT_MESH.f90,
                                         TYPHON_FMT.f90:95-170
  structured 2D generators (quad, tri)   CFDTOOLS/FileFormat/ty2dmesh.f90:612-744
"""
import ctypes as C
import struct
from dataclasses import dataclass, field

import numpy as np

from . import _capi

# element types (CFDTOOLS/Mesh/ELEMVTEX.f90:17-37)
ELEM_BAR2, ELEM_TRI3, ELEM_QUAD4, ELEM_TETRA4, ELEM_PENTA6, ELEM_HEXA8 = 2, 13, 24, 101, 131, 141
NVTEX = {ELEM_BAR2: 2, ELEM_TRI3: 3, ELEM_QUAD4: 4, ELEM_TETRA4: 4, ELEM_PENTA6: 6, ELEM_HEXA8: 8}
DIM = {ELEM_BAR2: 1, ELEM_TRI3: 2, ELEM_QUAD4: 2, ELEM_TETRA4: 3, ELEM_PENTA6: 3, ELEM_HEXA8: 3}

BC_PERIODIC, BC_SYMMETRY, BC_WALL, BC_FARFIELD, BC_NOSLIP, BC_HEAT = 1, 2, 3, 4, 5, 6
# inlets and outlets (parameters per face through Grid.set_boundary_params)
BC_INLET_SUB, BC_OUTLET_SUB, BC_INLET_SUP, BC_OUTLET_SUP = 7, 8, 9, 10


@dataclass
class RawMesh:
    vtex: np.ndarray                                   # (nvtex, 3) float64
    sections: list = field(default_factory=list)       # [(elemtype, ielem int32[n], conn int32[n, nv])]
    # [(family, tags int32[])]: face element numbers; [(family, tags, "vertex")]: vertex numbers
    marks: list = field(default_factory=list)

    @property
    def ncell(self):
        dmax = max(DIM[t] for t, _, _ in self.sections)
        return sum(len(ie) for t, ie, _ in self.sections if DIM[t] == dmax)


# ---------------------------------------------------------------------------
# XBIN / TYPHON format
_XBIN_HEADER = b"XBIN"


def _section_head(f, datatype, name, usertype, params=(), string=b""):
    f.write(struct.pack("<h", datatype))
    f.write(name.encode().ljust(32)[:32])
    f.write(struct.pack("<hhhhh", 0, usertype, 4, 8, len(params)))
    if params:
        f.write(np.asarray(params, dtype="<i4").tobytes())
    f.write(struct.pack("<h", len(string)))
    f.write(string)


def write_tym(path, raw: RawMesh):
    """Write a TYPHON mesh file (XBIN version 2, TYPHON format version 3).  Marks must be face
    element numbers (the format has no vertex marks)."""
    if any(len(m) > 2 and m[2] == "vertex" for m in raw.marks):
        raise ValueError("vertex-located boundary marks cannot be written to a .tym file")
    cells = [s for s in raw.sections if DIM[s[0]] == max(DIM[t] for t, _, _ in raw.sections)]
    faces = [s for s in raw.sections if s not in cells]
    with open(path, "wb") as f:
        f.write(_XBIN_HEADER + bytes([0, 2]) + bytes([4, 3, 2, 1]))
        _section_head(f, 1, "FILE_HEADER", 1, (3, 10, 1, 0, 11))
        f.write(b"END")
        ncell = sum(len(s[1]) for s in cells)
        nface = sum(len(s[1]) for s in faces)
        _section_head(f, 1, "USTMESH", 10, (0, ncell, nface, len(raw.vtex), len(cells), len(faces), 0,
                                             len(raw.marks)))
        f.write(b"END")
        for typ, ielem, conn in cells:
            _section_head(f, 15, "CELLS", 12, (typ,))
            f.write(struct.pack("<ii", len(ielem), NVTEX[typ]))
            f.write(np.asarray(ielem, "<i4").tobytes())
            f.write(np.asarray(conn, "<i4").tobytes())
            f.write(b"END")
        _section_head(f, 20, "NODES", 11)
        f.write(struct.pack("<iii", 1, len(raw.vtex), 3))
        f.write(np.asarray(raw.vtex, "<f8").tobytes())
        f.write(b"END")
        for typ, ielem, conn in faces:
            _section_head(f, 15, "FACES", 15, (typ,))
            f.write(struct.pack("<ii", len(ielem), NVTEX[typ]))
            f.write(np.asarray(ielem, "<i4").tobytes())
            f.write(np.asarray(conn, "<i4").tobytes())
            f.write(b"END")
        for name, tags, *_ in raw.marks:
            _section_head(f, 10, name, 20)
            f.write(struct.pack("<iii", 1, len(tags), 0))
            f.write(np.asarray(tags, "<i4").tobytes())
            f.write(b"END")


class _Reader:
    def __init__(self, data):
        self.d = data
        self.p = 0

    def take(self, n):
        if self.p + n > len(self.d):
            raise ValueError("truncated XBIN file")
        b = self.d[self.p:self.p + n]
        self.p += n
        return b

    def i16(self):
        return struct.unpack("<h", self.take(2))[0]

    def i32(self, n=1):
        v = np.frombuffer(self.take(4 * n), "<i4")
        return int(v[0]) if n == 1 else v.copy()

    def head(self, version):
        h = dict(datatype=self.i16(), name=self.take(32).decode().rstrip(" \0"))
        h["groupindex"], h["usertype"], h["intsize"], h["realsize"] = (self.i16() for _ in range(4))
        n = self.i16()
        h["param"] = [int(x) for x in np.atleast_1d(self.i32(n))] if n > 0 else []
        h["string"] = ""
        if version >= 2:
            sl = self.i16()
            h["string"] = self.take(sl).decode() if sl > 0 else ""
        if h["intsize"] != 4 or h["realsize"] != 8:
            raise ValueError("unexpected integer/real size in XBIN section " + h["name"])
        if h["datatype"] in (10, 20):
            h["firstindex"], h["nelem"], h["dim"] = self.i32(), self.i32(), self.i32()
        elif h["datatype"] in (15, 25):
            h["nelem"], h["dim"] = self.i32(), self.i32()
        return h

    def end(self):
        if self.take(3) != b"END":
            raise ValueError("bad end of XBIN data section")


def read_tym(path) -> RawMesh:
    """Read a TYPHON mesh file (little-endian XBIN, mesh_full)."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    if r.take(4) != _XBIN_HEADER:
        raise ValueError("not a XBIN file")
    v = r.take(2)
    version = v[0] * 256 + v[1]
    if r.take(4) != bytes([4, 3, 2, 1]):
        raise ValueError("only little-endian XBIN files are supported")
    h = r.head(version)
    r.end()
    ty_version = h["param"][0]
    mh = r.head(version)
    r.end()
    p = mh["param"]
    if ty_version == 1:
        ncellsec, nfacesec, nmark = p[4], p[5], p[6]
    else:
        ncellsec, nfacesec, nmark = p[4], p[5], p[7]
    if mh["string"]:
        raise ValueError("shared meshes are not supported")

    def elems(usertype):
        eh = r.head(version)
        if eh["usertype"] != usertype:
            raise ValueError("unexpected section " + eh["name"])
        typ, n, nv = eh["param"][0], eh["nelem"], eh["dim"]
        if eh["datatype"] == 15:
            ielem = r.i32(n) if n > 1 else np.array([r.i32()], np.int32)
        else:
            ielem = np.arange(eh["firstindex"], eh["firstindex"] + n, dtype=np.int32)
        conn = np.frombuffer(r.take(4 * n * nv), "<i4").reshape(n, nv).copy()
        r.end()
        return typ, np.asarray(ielem, np.int32), conn

    raw = RawMesh(vtex=np.zeros((0, 3)))
    for _ in range(ncellsec):
        raw.sections.append(elems(12))
    nh = r.head(version)
    raw.vtex = np.frombuffer(r.take(8 * nh["nelem"] * nh["dim"]), "<f8").reshape(nh["nelem"], nh["dim"]).copy()
    r.end()
    for _ in range(nfacesec):
        raw.sections.append(elems(15))
    for _ in range(nmark):
        mh2 = r.head(version)
        tags = np.frombuffer(r.take(4 * mh2["nelem"]), "<i4").copy()
        r.end()
        raw.marks.append((mh2["name"], tags))
    return raw


# ---------------------------------------------------------------------------
# Generators
def gen_grid2d(ni, nj, lx, ly, kind="tri", jitter=0.0, seed=1234):
    """Structured 2D grid on [0,lx]x[0,ly] in the numbering of ty2dmesh (ty2dmesh.f90:612-744).

    kind: "quad" (QUAD4) or "tri" (each quad split into (a,c,b) and (b,c,d)).  jitter moves
    every interior node by U(-jitter*h, +jitter*h) in x and y (numpy default_rng(seed));
    boundary nodes stay on the box so that periodic faces match.  Marks: IMIN, IMAX, JMIN,
    JMAX (BAR2 face elements numbered 1..2(ni+nj)).
    """
    i = np.arange(ni + 1)[:, None]
    j = np.arange(nj + 1)[None, :]
    hx, hy = lx / ni, ly / nj
    x = np.broadcast_to(i * hx, (ni + 1, nj + 1)).astype(np.float64).copy()
    y = np.broadcast_to(j * hy, (ni + 1, nj + 1)).astype(np.float64).copy()
    if jitter > 0:
        rng = np.random.default_rng(seed)
        dx = rng.uniform(-jitter * hx, jitter * hx, size=(ni + 1, nj + 1))
        dy = rng.uniform(-jitter * hy, jitter * hy, size=(ni + 1, nj + 1))
        inner = np.zeros((ni + 1, nj + 1), bool)
        inner[1:-1, 1:-1] = True
        x[inner] += dx[inner]
        y[inner] += dy[inner]
    vtex = np.stack([x.reshape(-1), y.reshape(-1), np.zeros((ni + 1) * (nj + 1))], axis=1)
    I, J = np.meshgrid(np.arange(1, ni + 1), np.arange(1, nj + 1), indexing="ij")
    I, J = I.reshape(-1), J.reshape(-1)
    iva = (I - 1) * (nj + 1) + J
    ivb, ivc, ivd = iva + 1, iva + (nj + 1), iva + 1 + (nj + 1)
    if kind == "quad":
        conn = np.stack([iva, ivc, ivd, ivb], axis=1).astype(np.int32)
        sec = (ELEM_QUAD4, np.arange(1, ni * nj + 1, dtype=np.int32), conn)
    else:
        conn = np.empty((2 * ni * nj, 3), np.int32)
        conn[0::2] = np.stack([iva, ivc, ivb], axis=1)
        conn[1::2] = np.stack([ivb, ivc, ivd], axis=1)
        sec = (ELEM_TRI3, np.arange(1, 2 * ni * nj + 1, dtype=np.int32), conn)
    jj = np.arange(1, nj + 1)
    ii = np.arange(1, ni + 1)
    bar_imin = np.stack([jj, jj + 1], 1)
    base = ni * (nj + 1)
    bar_imax = np.stack([base + jj, base + jj + 1], 1)
    bar_jmin = np.stack([(ii - 1) * (nj + 1) + 1, ii * (nj + 1) + 1], 1)
    bar_jmax = np.stack([ii * (nj + 1), (ii + 1) * (nj + 1)], 1)
    bars = np.concatenate([bar_imin, bar_imax, bar_jmin, bar_jmax]).astype(np.int32)
    nb = len(bars)
    fsec = (ELEM_BAR2, np.arange(1, nb + 1, dtype=np.int32), bars)
    marks = [("IMIN", np.arange(1, nj + 1, dtype=np.int32)),
             ("IMAX", np.arange(nj + 1, 2 * nj + 1, dtype=np.int32)),
             ("JMIN", np.arange(2 * nj + 1, 2 * nj + ni + 1, dtype=np.int32)),
             ("JMAX", np.arange(2 * nj + ni + 1, 2 * (nj + ni) + 1, dtype=np.int32))]
    return RawMesh(vtex=vtex, sections=[sec, fsec], marks=marks)


def gen_tet_box(n, length, jitter=0.0, seed=1234):
    """n^3 hexahedra on [0,length]^3, each split into 5 tetrahedra with alternating parity
    (conforming, also across periodic boundaries for even n); interior nodes jittered by
    U(-jitter*h, +jitter*h) per coordinate (numpy default_rng(seed)).  Boundary triangles
    are marked IMIN/IMAX (x), JMIN/JMAX (y), KMIN/KMAX (z)."""
    h = length / n
    g = np.arange(n + 1) * h
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    vt = np.stack([X, Y, Z], axis=-1).reshape(-1, 3).astype(np.float64)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter * h, jitter * h, size=vt.shape)
        idx = np.arange(n + 1)
        inner = ((idx[:, None, None] > 0) & (idx[:, None, None] < n) &
                 (idx[None, :, None] > 0) & (idx[None, :, None] < n) &
                 (idx[None, None, :] > 0) & (idx[None, None, :] < n)).reshape(-1)
        vt[inner] += d[inner]

    def vid(i, j, k):
        return (i * (n + 1) + j) * (n + 1) + k + 1

    I, J, K = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    I, J, K = I.reshape(-1), J.reshape(-1), K.reshape(-1)
    v = [vid(I, J, K), vid(I + 1, J, K), vid(I + 1, J + 1, K), vid(I, J + 1, K),
         vid(I, J, K + 1), vid(I + 1, J, K + 1), vid(I + 1, J + 1, K + 1), vid(I, J + 1, K + 1)]
    v = np.stack(v, axis=1)
    even = ((I + J + K) % 2 == 0)[:, None]
    tets_even = [(1, 3, 4, 6), (0, 1, 3, 4), (2, 3, 1, 6), (5, 4, 6, 1), (7, 6, 4, 3)]
    tets_odd = [(0, 2, 5, 7), (1, 0, 2, 5), (3, 2, 0, 7), (4, 5, 7, 0), (6, 7, 5, 2)]
    conn = np.empty((len(I), 5, 4), np.int32)
    for t in range(5):
        conn[:, t, :] = np.where(even, v[:, list(tets_even[t])], v[:, list(tets_odd[t])])
    conn = conn.reshape(-1, 4)
    # boundary triangles: the element faces whose three nodes lie on one face of the box (the
    # faces seen once), in element-face order; only the tetrahedra of the outer hexahedron
    # layer can own one
    layer = ((I == 0) | (I == n - 1) | (J == 0) | (J == n - 1) | (K == 0) | (K == n - 1))
    outer = conn[np.repeat(layer, 5)]
    fl = np.concatenate([outer[:, [0, 2, 1]], outer[:, [0, 1, 3]], outer[:, [1, 2, 3]], outer[:, [2, 0, 3]]])
    ijk = np.unravel_index(fl - 1, (n + 1, n + 1, n + 1))
    on = np.zeros(len(fl), bool)
    for a in range(3):
        on |= (ijk[a] == 0).all(axis=1) | (ijk[a] == n).all(axis=1)
    bnd = fl[on]
    cen = vt[bnd - 1].mean(axis=1)
    tol = 1e-9 * length
    names = [("IMIN", 0, 0.0), ("IMAX", 0, length), ("JMIN", 1, 0.0), ("JMAX", 1, length),
             ("KMIN", 2, 0.0), ("KMAX", 2, length)]
    faces, marks, nextid = [], [], 1
    for name, ax, val in names:
        sel = bnd[np.abs(cen[:, ax] - val) < tol]
        ids = np.arange(nextid, nextid + len(sel), dtype=np.int32)
        nextid += len(sel)
        faces.append(sel)
        marks.append((name, ids))
    fconn = np.concatenate(faces).astype(np.int32)
    secs = [(ELEM_TETRA4, np.arange(1, len(conn) + 1, dtype=np.int32), conn),
            (ELEM_TRI3, np.arange(1, len(fconn) + 1, dtype=np.int32), fconn)]
    return RawMesh(vtex=vt, sections=secs, marks=marks)


def gen_flatplate(nx=200, nz=20, n_prism=50, n_tet=25, x0=-0.5, x1=1.0, width=0.2, y1=1.74e-3, growth=1.1):
    """Flat-plate box: prisms stretched to the plate, tetrahedra above.

    The (x, z) plane [x0, x1] x [0, width] carries nx x nz quadrilaterals, each split along
    its (i, k)-(i+1, k+1) diagonal into two triangles.  The triangles are extruded in y into
    n_prism layers of prisms (PENTA6), the first layer y1 thick, each layer `growth` times the
    previous one.  Above, n_tet layers of hexahedra as thick as the last prism layer are split
    into 6 tetrahedra each (the Kuhn split along the (0,0,0)-(1,1,1) diagonal, which cuts
    every hexahedron face along its lowest-to-highest-corner diagonal, so the tetrahedra
    conform with each other and with the prisms' top triangles).  Cells: 2 nx nz n_prism
    prisms + 6 nx nz n_tet tetrahedra.

    Boundary marks: WALL (y = 0, x >= 0), UPSTREAM (y = 0, x < 0), INLET (x = x0),
    OUTLET (x = x1), TOP (y = top), SIDE0 / SIDE1 (z = 0 / width)."""
    yp = y1 * (growth ** np.arange(n_prism + 1) - 1.0) / (growth - 1.0)
    dyl = yp[-1] - yp[-2]
    y = np.concatenate([yp, yp[-1] + dyl * np.arange(1, n_tet + 1)])
    ny = len(y) - 1
    xs = np.linspace(x0, x1, nx + 1)
    zs = np.linspace(0.0, width, nz + 1)
    X, Y, Z = np.meshgrid(xs, y, zs, indexing="ij")
    vt = np.stack([X, Y, Z], axis=-1).reshape(-1, 3).astype(np.float64)

    def vid(i, j, k):
        return (i * (ny + 1) + j) * (nz + 1) + k + 1

    # prisms: triangles (i,k)(i+1,k)(i+1,k+1) and (i,k)(i+1,k+1)(i,k+1), layer j -> j+1
    I, J, K = np.meshgrid(np.arange(nx), np.arange(n_prism), np.arange(nz), indexing="ij")
    I, J, K = I.reshape(-1), J.reshape(-1), K.reshape(-1)
    tri = [((0, 0), (1, 0), (1, 1)), ((0, 0), (1, 1), (0, 1))]
    prisms = []
    for t in tri:
        bot = [vid(I + a, J, K + b) for a, b in t]
        top = [vid(I + a, J + 1, K + b) for a, b in t]
        prisms.append(np.stack(bot + top, axis=1))
    prisms = np.stack(prisms, axis=1).reshape(-1, 6).astype(np.int32)
    # tetrahedra: Kuhn split of hexahedra j = n_prism .. ny-1
    I, J, K = np.meshgrid(np.arange(nx), np.arange(n_prism, ny), np.arange(nz), indexing="ij")
    I, J, K = I.reshape(-1), J.reshape(-1), K.reshape(-1)
    tets = []
    axes = {"x": (1, 0, 0), "y": (0, 1, 0), "z": (0, 0, 1)}
    for perm in ("xyz", "xzy", "yxz", "yzx", "zxy", "zyx"):
        p0 = np.zeros(3, int)
        path = [p0.copy()]
        for a in perm[:2]:
            p0 = p0 + np.array(axes[a])
            path.append(p0.copy())
        path.append(np.array((1, 1, 1)))
        tets.append(np.stack([vid(I + d[0], J + d[1], K + d[2]) for d in path], axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    # positive orientation for every tetrahedron
    a, b, c, d = (vt[tets[:, q] - 1] for q in range(4))
    neg = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a) < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    # boundary faces: faces seen once
    ptri = np.concatenate([prisms[:, [0, 1, 2]], prisms[:, [3, 4, 5]]])
    pquad = np.concatenate([prisms[:, [0, 2, 5, 3]], prisms[:, [0, 1, 4, 3]], prisms[:, [1, 2, 5, 4]]])
    ttri = np.concatenate([tets[:, [0, 2, 1]], tets[:, [0, 1, 3]], tets[:, [1, 2, 3]], tets[:, [2, 0, 3]]])
    alltri = np.concatenate([ptri, ttri])

    def once(f):
        # on a box the faces seen once are those whose nodes all lie on one of its six planes
        ijk = np.unravel_index(f - 1, (nx + 1, ny + 1, nz + 1))
        on = np.zeros(len(f), bool)
        for a, top_index in enumerate((nx, ny, nz)):
            on |= (ijk[a] == 0).all(axis=1) | (ijk[a] == top_index).all(axis=1)
        return f[on]

    btri, bquad = once(alltri), once(pquad)
    top = y[-1]
    tol = 1e-9

    def classify(f):
        c = vt[f - 1].mean(axis=1)
        lab = np.full(len(f), "", dtype=object)
        lab[np.abs(c[:, 2]) < tol] = "SIDE0"
        lab[np.abs(c[:, 2] - width) < tol] = "SIDE1"
        lab[np.abs(c[:, 0] - x0) < tol] = "INLET"
        lab[np.abs(c[:, 0] - x1) < tol] = "OUTLET"
        lab[np.abs(c[:, 1] - top) < tol] = "TOP"
        lab[(np.abs(c[:, 1]) < tol) & (c[:, 0] >= 0.0)] = "WALL"
        lab[(np.abs(c[:, 1]) < tol) & (c[:, 0] < 0.0)] = "UPSTREAM"
        assert (lab != "").all()
        return lab

    lt, lq = classify(btri), classify(bquad)
    nt = len(btri)
    marks = []
    for name in ("WALL", "UPSTREAM", "INLET", "OUTLET", "TOP", "SIDE0", "SIDE1"):
        ids = np.concatenate([np.nonzero(lt == name)[0] + 1, nt + np.nonzero(lq == name)[0] + 1]).astype(np.int32)
        marks.append((name, ids))
    ncp = len(prisms)
    secs = [(ELEM_PENTA6, np.arange(1, ncp + 1, dtype=np.int32), prisms),
            (ELEM_TETRA4, np.arange(ncp + 1, ncp + len(tets) + 1, dtype=np.int32), tets),
            (ELEM_TRI3, np.arange(1, nt + 1, dtype=np.int32), btri.astype(np.int32)),
            (ELEM_QUAD4, np.arange(nt + 1, nt + len(bquad) + 1, dtype=np.int32), bquad.astype(np.int32))]
    return RawMesh(vtex=vt, sections=secs, marks=marks)


def gen_kuhn_box(n, length=1.0):
    """n^3 hexahedra on [0, length]^3, each split into 6 tetrahedra along its
    (0,0,0)-(1,1,1) diagonal (the Kuhn split: conforming, every face cut along its
    lowest-to-highest-corner diagonal).  Boundary triangles are marked IMIN/IMAX (x),
    JMIN/JMAX (y), KMIN/KMAX (z)."""
    g = np.arange(n + 1) * (length / n)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    vt = np.stack([X, Y, Z], axis=-1).reshape(-1, 3).astype(np.float64)

    def vid(i, j, k):
        return (i * (n + 1) + j) * (n + 1) + k + 1

    I, J, K = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    I, J, K = I.reshape(-1), J.reshape(-1), K.reshape(-1)
    axes = {"x": (1, 0, 0), "y": (0, 1, 0), "z": (0, 0, 1)}
    tets = []
    for perm in ("xyz", "xzy", "yxz", "yzx", "zxy", "zyx"):
        p0 = np.zeros(3, int)
        path = [p0.copy()]
        for a in perm[:2]:
            p0 = p0 + np.array(axes[a])
            path.append(p0.copy())
        path.append(np.array((1, 1, 1)))
        tets.append(np.stack([vid(I + d[0], J + d[1], K + d[2]) for d in path], axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    a, b, c, d = (vt[tets[:, q] - 1] for q in range(4))
    neg = np.einsum("ij,ij->i", np.cross(b - a, c - a), d - a) < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    # boundary triangles: the element faces whose three nodes lie on one face of the box (the
    # faces seen once), in element-face order; only the tetrahedra of the outer hexahedron
    # layer can own one
    layer = ((I == 0) | (I == n - 1) | (J == 0) | (J == n - 1) | (K == 0) | (K == n - 1))
    outer = tets[np.repeat(layer, 6)]
    fl = np.concatenate([outer[:, [0, 2, 1]], outer[:, [0, 1, 3]], outer[:, [1, 2, 3]], outer[:, [2, 0, 3]]])
    ijk = np.unravel_index(fl - 1, (n + 1, n + 1, n + 1))
    on = np.zeros(len(fl), bool)
    for a in range(3):
        on |= (ijk[a] == 0).all(axis=1) | (ijk[a] == n).all(axis=1)
    bnd = fl[on]
    cen = vt[bnd - 1].mean(axis=1)
    tol = 1e-9 * length
    faces, marks, nextid = [], [], 1
    for name, ax, v in (("IMIN", 0, 0.0), ("IMAX", 0, length), ("JMIN", 1, 0.0), ("JMAX", 1, length),
                        ("KMIN", 2, 0.0), ("KMAX", 2, length)):
        sel = bnd[np.abs(cen[:, ax] - v) < tol]
        faces.append(sel)
        marks.append((name, np.arange(nextid, nextid + len(sel), dtype=np.int32)))
        nextid += len(sel)
    fconn = np.concatenate(faces).astype(np.int32)
    secs = [(ELEM_TETRA4, np.arange(1, len(tets) + 1, dtype=np.int32), tets),
            (ELEM_TRI3, np.arange(1, len(fconn) + 1, dtype=np.int32), fconn)]
    return RawMesh(vtex=vt, sections=secs, marks=marks)


def flatplate_bcs(wall_velocity=(0.0, 0.0, 0.0)):
    """Adiabatic no-slip plate, symmetry upstream of it and on the span sides, far field
    at the inlet, outlet and top."""
    return [("WALL", BC_NOSLIP, "", (0.0, 0.0, 0.0), tuple(wall_velocity)),
            ("UPSTREAM", BC_SYMMETRY, "", (0.0, 0.0, 0.0)),
            ("SIDE0", BC_SYMMETRY, "", (0.0, 0.0, 0.0)), ("SIDE1", BC_SYMMETRY, "", (0.0, 0.0, 0.0)),
            ("INLET", BC_FARFIELD, "", (0.0, 0.0, 0.0)), ("OUTLET", BC_FARFIELD, "", (0.0, 0.0, 0.0)),
            ("TOP", BC_FARFIELD, "", (0.0, 0.0, 0.0))]


# ---------------------------------------------------------------------------
def periodic_box_bcs(lengths):
    """Periodic connections IMIN<->IMAX, JMIN<->JMAX (and KMIN<->KMAX in 3D)."""
    out = [("IMIN", BC_PERIODIC, "IMAX", (lengths[0], 0.0, 0.0)),
           ("JMIN", BC_PERIODIC, "JMAX", (0.0, lengths[1], 0.0))]
    if len(lengths) > 2:
        out.append(("KMIN", BC_PERIODIC, "KMAX", (0.0, 0.0, lengths[2])))
    return out


class MeshDesc:
    """Preprocessed mesh (numpy copies of the ty_mesh_desc arrays, 0-based where noted)."""

    def __init__(self, d, facevtex, face_family=None, families=()):
        nf, nc = d.nface, d.ncell

        def arr(ptr, n, dt):
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(dt)), shape=(n,)).copy()

        self.dim, self.ncell_int, self.ncell = d.dim, d.ncell_int, d.ncell
        self.nface_int, self.nface = d.nface_int, d.nface
        self.facecell = arr(d.facecell, 2 * nf, C.c_int32)          # 1-based, fils(nf,2)
        self.face_normal = arr(d.face_normal, 3 * nf, C.c_double).reshape(nf, 3)
        self.face_surface = arr(d.face_surface, nf, C.c_double)
        self.face_centre = arr(d.face_centre, 3 * nf, C.c_double).reshape(nf, 3)
        self.cell_centre = arr(d.cell_centre, 3 * nc, C.c_double).reshape(nc, 3)
        self.cell_volume = arr(d.cell_volume, nc, C.c_double)
        self.face_color = arr(d.face_color, nf, C.c_int32)
        self.face_bc = arr(d.face_bc, nf, C.c_int32)
        self.face_partner = arr(d.face_partner, nf, C.c_int32)      # 1-based, 0 = none
        self.face_wallvel = arr(d.face_wallvel, 3 * nf, C.c_double).reshape(nf, 3)
        self.facevtex = facevtex
        # boundary definition index of each face (bcs order given to preprocess), -1 interior
        self.face_family = face_family if face_family is not None else np.full(nf, -1, np.int32)
        self.families = list(families)
        # [nface, 3, 3] rotation into each face's frame when a periodic family is rotational
        self.face_rotation = None

    def faces_of(self, family):
        """Faces (0-based) of a boundary family, in face order."""
        return np.nonzero(self.face_family == self.families.index(family.upper()))[0]

    @property
    def fc1(self):
        return self.facecell[:self.nface] - 1

    @property
    def fc2(self):
        return self.facecell[self.nface:] - 1

    def to_c(self):
        """A ty_mesh_desc pointing into this object's arrays (keep the object alive)."""
        for k in ("facecell", "face_color", "face_bc", "face_partner"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.int32))
        for k in ("face_normal", "face_surface", "face_centre", "cell_centre", "cell_volume", "face_wallvel"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float64))
        d = _capi.MeshDesc()
        d.dim, d.ncell_int, d.ncell, d.nface_int, d.nface = (self.dim, self.ncell_int, self.ncell,
                                                             self.nface_int, self.nface)
        for k in ("facecell", "face_normal", "face_surface", "face_centre", "cell_centre", "cell_volume",
                  "face_color", "face_bc", "face_partner", "face_wallvel"):
            setattr(d, k, getattr(self, k).ctypes.data)
        return d


def _umesh_built(L, raw: RawMesh, dim, bcs, rotations):
    """A ty_umesh handle holding raw, bcs and rotations, built (the caller frees it)."""
    h = C.c_void_p()
    _capi.check(L.ty_umesh_new(C.byref(h)), "ty_umesh_new")
    try:
        vt = np.ascontiguousarray(raw.vtex, np.float64)
        _capi.check(L.ty_umesh_set_nodes(h, vt.shape[0], vt.ctypes.data), "ty_umesh_set_nodes")
        for typ, ielem, conn in raw.sections:
            ie = np.ascontiguousarray(ielem, np.int32)
            cv = np.ascontiguousarray(conn, np.int32)
            _capi.check(L.ty_umesh_add_section(h, int(typ), ie.shape[0], ie.ctypes.data, cv.ctypes.data),
                        "ty_umesh_add_section")
        for name, tags, *loc in raw.marks:
            t = np.ascontiguousarray(tags, np.int32)
            if loc and loc[0] == "vertex":
                _capi.check(L.ty_umesh_add_vertex_mark(h, name.encode(), t.shape[0], t.ctypes.data),
                            "ty_umesh_add_vertex_mark")
            else:
                _capi.check(L.ty_umesh_add_mark(h, name.encode(), t.shape[0], t.ctypes.data), "ty_umesh_add_mark")
        for b in bcs:
            tr = np.ascontiguousarray(b[3] if len(b) > 3 and b[3] is not None else (0, 0, 0), np.float64)
            wv = np.ascontiguousarray(b[4] if len(b) > 4 else (0, 0, 0), np.float64)
            _capi.check(L.ty_umesh_add_bc(h, b[0].encode(), int(b[1]), (b[2] or "").encode(),
                                          tr.ctypes.data, wv.ctypes.data), "ty_umesh_add_bc")
        for fam, (ctr, ax, ang) in (rotations or {}).items():
            c3 = np.ascontiguousarray(ctr, np.float64)
            a3 = np.ascontiguousarray(ax, np.float64)
            _capi.check(L.ty_umesh_set_rotation(h, fam.encode(), c3.ctypes.data, a3.ctypes.data, float(ang)),
                        "ty_umesh_set_rotation")
        _capi.check(L.ty_umesh_build(h, int(dim)), "ty_umesh_build")
    except BaseException:
        L.ty_umesh_free(h)
        raise
    return h


def preprocess(raw: RawMesh, dim, bcs, rotations=None) -> MeshDesc:
    """Native preprocessing (ty_umesh_*): faces, geometry, colours, ghosts, periodicity.

    bcs: [(family, kind, partner, translation(3)[, wall_velocity(3)])]
    rotations: {family: (centre(3), axis(3), angle in degrees)} for periodic families that
    are connected to their partner by a rotation (BLOCK:PERIODICITY TYPE = ROTATION)
    """
    L = _capi.lib()
    h = _umesh_built(L, raw, dim, bcs, rotations)
    try:
        d = _capi.MeshDesc()
        _capi.check(L.ty_umesh_desc(h, C.byref(d)), "ty_umesh_desc")
        fv = np.zeros(4 * d.nface, np.int32)
        _capi.check(L.ty_umesh_facevtex(h, fv.ctypes.data), "ty_umesh_facevtex")
        ff = np.zeros(d.nface, np.int32)
        _capi.check(L.ty_umesh_face_family(h, ff.ctypes.data), "ty_umesh_face_family")
        md = MeshDesc(d, fv.reshape(d.nface, 4), ff, [b[0].upper() for b in bcs])
        if rotations:                                 # [nface][3][3] only when a family rotates
            rot = np.zeros(9 * d.nface)
            rc = L.ty_umesh_face_rotation(h, rot.ctypes.data)
            _capi.check(min(rc, 0), "ty_umesh_face_rotation")
            if rc == 1:
                md.face_rotation = rot.reshape(d.nface, 3, 3)
        return md
    finally:
        L.ty_umesh_free(h)


def reorder_rcm(raw: RawMesh, dim, bcs, rotations=None) -> RawMesh:
    """The same mesh with the element rows of each cell section in reverse Cuthill-McKee
    order (ty_umesh_rcm_order; element numbers, nodes and boundary marks unchanged), so that
    preprocessing it numbers neighbouring cells, and the faces made from them, close together.
    Typhon keeps the file's order; this is the locality renumbering applied before
    preprocessing, for meshes whose native numbering scatters neighbours."""
    L = _capi.lib()
    h = _umesh_built(L, raw, dim, bcs, rotations)
    try:
        order = np.zeros(raw.ncell, np.int32)
        _capi.check(L.ty_umesh_rcm_order(h, order.ctypes.data), "ty_umesh_rcm_order")
    finally:
        L.ty_umesh_free(h)
    dmax = max(DIM[t] for t, _, _ in raw.sections)
    secs, off = [], 0
    for typ, ielem, conn in raw.sections:
        if DIM[typ] == dmax:
            m = len(ielem)
            secs.append((typ, np.asarray(ielem, np.int32).copy(), np.ascontiguousarray(conn[order[off:off + m]])))
            off += m
        else:
            secs.append((typ, ielem, conn))
    return RawMesh(vtex=raw.vtex, sections=secs, marks=list(raw.marks))
