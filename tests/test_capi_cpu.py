"""CPU checks of the C ABI library: it loads, exports every declared entry point, its
native mesh preprocessing reproduces Typhon's (the oracle's) arrays bit for bit, the
.tym reader/writer round-trips, and argument errors come back as status codes."""
import ctypes as C
import pathlib
import re

import numpy as np
import pytest

import oracle_py as op

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def ty():
    from typhon_gb300 import build
    build.build()
    import typhon_gb300
    return typhon_gb300


def declared_entry_points():
    text = (ROOT / "include" / "typhon_gpu.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(ty_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(ty):
    from typhon_gb300 import _capi
    lib = _capi.lib()
    names = declared_entry_points()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_capi.exported_names())
    assert lib.ty_version().decode().startswith("typhon_gb300")


def test_argument_errors_without_gpu(ty):
    from typhon_gb300 import _capi
    lib = _capi.lib()
    h = C.c_void_p()
    assert lib.ty_mesh_create(None, 0, C.byref(h)) == -1
    assert lib.ty_set_params(None, None) == -1
    assert lib.ty_error_string(-5).decode() == "negative or NaN internal energy"
    d = _capi.MeshDesc()
    d.dim = 4
    assert lib.ty_mesh_create(C.byref(d), 0, C.byref(h)) == -1


def _same(md, d):
    return {
        "fc1": np.array_equal(md.fc1, d["fc1"]), "fc2": np.array_equal(md.fc2, d["fc2"]),
        "normal": np.array_equal(md.face_normal, d["fnormal"]),
        "fcentre": np.array_equal(md.face_centre, d["fcentre"]),
        "surface": np.array_equal(md.face_surface, d["fsurf"]),
        "centre": np.array_equal(md.cell_centre, d["ccentre"]),
        "volume": np.array_equal(md.cell_volume, d["cvol"]),
        "colour": np.array_equal(md.face_color, d["face_color"]),
        "partner": np.array_equal(md.face_partner - 1, d["face_partner"]),
        "bc": np.array_equal(md.face_bc, d["face_bckind"]),
    }


def test_preprocess_quad20_matches_oracle(ty, golden_dir):
    raw = ty.read_tym(golden_dir / "quad20x20.tym")
    md = ty.preprocess(raw, 2, ty.periodic_box_bcs((1.0, 1.0)))
    d = op.Mesh.from_tym(golden_dir / "quad20x20.tym").build(2, op.PERIODIC_UNIT_SQUARE).export()
    assert all(_same(md, d).values()), _same(md, d)


def test_preprocess_symmetry_quad20x10_matches_oracle(ty, golden_dir):
    bcs = [(f, op.BC_SYMMETRY, "", (0, 0, 0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX")]
    raw = ty.read_tym(golden_dir / "quad20x10.tym")
    md = ty.preprocess(raw, 2, bcs)
    d = op.Mesh.from_tym(golden_dir / "quad20x10.tym").build(2, bcs).export()
    assert all(_same(md, d).values()), _same(md, d)


@pytest.mark.parametrize("n", [8, 64])
def test_preprocess_vortex_mesh_matches_oracle(ty, n):
    raw = ty.gen_grid2d(n, n, 10.0, 10.0, "tri", jitter=0.1, seed=1234)
    md = ty.preprocess(raw, 2, ty.periodic_box_bcs((10.0, 10.0)))
    d = op.Mesh.from_raw(raw).build(2, ty.periodic_box_bcs((10.0, 10.0))).export()
    assert all(_same(md, d).values()), _same(md, d)
    if n == 64:  # the configuration's sizes: 8192 triangles, 12416 faces, 256 periodic faces
        assert (md.ncell_int, md.nface, md.nface - md.nface_int) == (8192, 12416, 256)


@pytest.mark.parametrize("n", [4, 6])
def test_preprocess_tet_box_matches_oracle(ty, n):
    L = 2 * np.pi
    raw = ty.gen_tet_box(n, L, jitter=0.05, seed=1234)
    md = ty.preprocess(raw, 3, ty.periodic_box_bcs((L, L, L)))
    d = op.Mesh.from_raw(raw).build(3, ty.periodic_box_bcs((L, L, L))).export()
    assert all(_same(md, d).values()), _same(md, d)
    assert md.ncell_int == 5 * n ** 3
    assert abs(md.cell_volume[:md.ncell_int].sum() - L ** 3) < 1e-9 * L ** 3


def test_preprocess_flatplate_prisms_tets_matches_oracle(ty):
    """Mixed prism/tetrahedron mesh with wall, symmetry and far-field families."""
    raw = ty.umesh.gen_flatplate(nx=12, nz=3, n_prism=4, n_tet=3)
    bcs = ty.umesh.flatplate_bcs()
    md = ty.preprocess(raw, 3, bcs)
    d = op.Mesh.from_raw(raw).build(3, bcs).export()
    assert all(_same(md, d).values()), _same(md, d)
    assert md.ncell_int == 2 * 12 * 3 * 4 + 6 * 12 * 3 * 3
    assert np.all(md.cell_volume[:md.ncell_int] > 0)
    top = raw.vtex[:, 1].max()
    assert abs(md.cell_volume[:md.ncell_int].sum() - 1.5 * 0.2 * top) < 1e-12
    kinds = md.face_bc[md.nface_int:]
    assert set(np.unique(kinds)) == {ty.BC_NOSLIP, ty.BC_SYMMETRY, ty.BC_FARFIELD}


def test_tym_roundtrip(ty, tmp_path):
    raw = ty.gen_grid2d(6, 5, 3.0, 2.0, "quad")
    p = tmp_path / "m.tym"
    ty.write_tym(p, raw)
    back = ty.read_tym(p)
    assert np.array_equal(back.vtex, raw.vtex)
    for a, b in zip(back.sections, raw.sections):
        assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert [m[0] for m in back.marks] == [m[0] for m in raw.marks]
    # the oracle's independent reader agrees
    m = op.Mesh.from_tym(p).build(2, [("IMIN", op.BC_PERIODIC, "IMAX", (3.0, 0, 0)),
                                      ("JMIN", op.BC_PERIODIC, "JMAX", (0, 2.0, 0))])
    assert m.ncell_int == 30


def test_golden_mesh_reader_agrees(ty, golden_dir):
    for name in ("quad20x20.tym", "quad10x10.tym", "tri5x10.tym", "mxlay2x20quad-h50.tym"):
        raw = ty.read_tym(golden_dir / name)
        assert raw.ncell > 0 and raw.vtex.shape[1] == 3


def test_bad_mesh_is_rejected(ty):
    raw = ty.gen_grid2d(4, 4, 1.0, 1.0, "quad")
    with pytest.raises(ty.TyphonError):
        ty.preprocess(raw, 2, [("IMIN", 1, "IMAX", (1.0, 0, 0))])   # JMIN/JMAX undefined


def _faces_seen_once(sections):
    """Reference definition of the boundary: the element faces that belong to one element only."""
    from collections import Counter
    from typhon_gb300 import umesh
    local = {umesh.ELEM_TETRA4: [(0, 2, 1), (0, 1, 3), (1, 2, 3), (2, 0, 3)],
             umesh.ELEM_PENTA6: [(0, 1, 2), (3, 4, 5), (0, 2, 5, 3), (0, 1, 4, 3), (1, 2, 5, 4)]}
    cnt = Counter()
    for typ, _, conn in sections:
        for loc in local[typ]:
            for row in conn[:, list(loc)]:
                cnt[tuple(sorted(row))] += 1
    return {k for k, v in cnt.items() if v == 1}


@pytest.mark.parametrize("kind", ["tet", "kuhn", "plate"])
def test_generator_boundary_is_faces_seen_once(ty, kind):
    """The generators find their boundary triangles and quadrilaterals by a plane test on the
    box's grid indices; every boundary face is an element face seen once, and every element
    face seen once is marked exactly once."""
    if kind == "tet":
        raw = ty.umesh.gen_tet_box(4, 1.0, jitter=0.05, seed=3)
    elif kind == "kuhn":
        raw = ty.umesh.gen_kuhn_box(3, 1.0)
    else:
        raw = ty.umesh.gen_flatplate(nx=6, nz=2, n_prism=3, n_tet=2)
    cell_types = (ty.umesh.ELEM_TETRA4, ty.umesh.ELEM_PENTA6)
    cells = [s for s in raw.sections if s[0] in cell_types]
    faces = [s for s in raw.sections if s[0] not in cell_types]
    bnd = [tuple(sorted(r)) for _, _, conn in faces for r in conn]
    assert len(bnd) == len(set(bnd))
    assert set(bnd) == _faces_seen_once(cells)
    marked = np.sort(np.concatenate([m[1] for m in raw.marks]))
    assert np.array_equal(marked, np.arange(1, len(bnd) + 1))


def _neighbour_spread(md):
    nfi = md.nface_int
    c1, c2 = md.fc1[:nfi], md.fc2[:nfi]
    inner = c2 < md.ncell_int
    return float(np.abs(c1[inner] - c2[inner]).mean())


def test_rcm_order_restores_locality_and_keeps_oracle_parity(ty):
    """A tet box with its cells shuffled, renumbered in reverse Cuthill-McKee order: the mean
    index distance between face neighbours falls back to that of the generator's numbering,
    the cells are the same (a permutation of the element rows, element numbers in place), and
    the native preprocessing of the renumbered mesh is still the oracle's bit for bit."""
    from typhon_gb300 import cases
    L = 2 * np.pi
    raw = ty.gen_tet_box(10, L, jitter=0.05, seed=1234)
    bcs = ty.periodic_box_bcs((L, L, L))
    mixed = cases.shuffle_cells(raw, seed=3)
    rcm = ty.reorder_rcm(mixed, 3, bcs)
    (t0, ie0, c0), (t1, ie1, c1) = mixed.sections[0], rcm.sections[0]
    assert t0 == t1 and np.array_equal(ie0, ie1)
    assert sorted(map(tuple, np.sort(c0, axis=1))) == sorted(map(tuple, np.sort(c1, axis=1)))
    md_mixed, md_rcm, md_gen = (ty.preprocess(r, 3, bcs) for r in (mixed, rcm, raw))
    assert _neighbour_spread(md_rcm) < 0.1 * _neighbour_spread(md_mixed)
    assert _neighbour_spread(md_rcm) < 2.0 * _neighbour_spread(md_gen)
    assert abs(md_rcm.cell_volume[:md_rcm.ncell_int].sum() - L ** 3) < 1e-9 * L ** 3
    d = op.Mesh.from_raw(rcm).build(3, bcs).export()
    assert all(_same(md_rcm, d).values()), _same(md_rcm, d)


def test_rcm_order_per_section(ty):
    """Prisms and tetrahedra are renumbered within their own sections."""
    raw = ty.umesh.gen_flatplate(nx=8, nz=2, n_prism=3, n_tet=2)
    bcs = ty.umesh.flatplate_bcs()
    rcm = ty.reorder_rcm(raw, 3, bcs)
    for (ta, ia, ca), (tb, ib, cb) in zip(raw.sections, rcm.sections):
        assert ta == tb and np.array_equal(ia, ib)
        assert sorted(map(tuple, np.sort(ca, axis=1))) == sorted(map(tuple, np.sort(cb, axis=1)))
    md = ty.preprocess(rcm, 3, bcs)
    d = op.Mesh.from_raw(rcm).build(3, bcs).export()
    assert all(_same(md, d).values()), _same(md, d)
