"""CGNS (ADF) meshes and Typhon's heat-conduction golden runs, without a GPU.

* typhon_gb300.cgns reads the CGNS meshes of Typhon's non-regression suite: a big-endian
  file with vertex-located boundary conditions (tube.cgns) and little-endian files with
  face-element ones (square-quad10.cgns, rect4x1.cgns); the native preprocessing and the
  oracle's agree face by face on them.
* The oracle's restatement of Typhon's steady implicit KDIF run (DLU matrix, cycles,
  residual, VOL_AVERAGE probe) with each of Typhon's DLU solvers (dlu_cgs, dlu_bicg,
  dlu_gmres) reproduces NRG/KDIF/ISOTH-CGS, -BICG and -GMRES: the 929 residuals of monres.001
  to 1e-10 in log10 (the files print 15 digits) and the five cycle averages of
  Average_T.tmon as printed (8 digits).
"""
import numpy as np
import pytest

import oracle_py as op
import typhon_gb300 as ty
from typhon_gb300 import cgns, umesh

TUBE_BCS = [("SYM", umesh.BC_HEAT, "", (0, 0, 0)), ("INFINI", umesh.BC_HEAT, "", (0, 0, 0)),
            ("WALL", umesh.BC_HEAT, "", (0, 0, 0))]


def test_reads_big_endian_vertex_bc_mesh(golden_dir):
    raw = cgns.read_cgns(golden_dir / "tube.cgns")
    assert raw.vtex.shape == (18, 3)
    assert [(t, len(ie)) for t, ie, _ in raw.sections] == [(umesh.ELEM_QUAD4, 10), (umesh.ELEM_BAR2, 14)]
    assert [(m[0], len(m[1]), m[2]) for m in raw.marks] == [("SYM", 12, "vertex"), ("INFINI", 3, "vertex"),
                                                           ("WALL", 3, "vertex")]
    assert raw.vtex[:, 0].min() == 0.0 and raw.vtex[:, 0].max() == 100.0 and raw.vtex[:, 1].max() == 10.0
    md = ty.preprocess(raw, 2, TUBE_BCS)
    assert (md.ncell_int, md.nface, md.nface_int) == (10, 27, 13)
    assert [len(md.faces_of(f)) for f in ("SYM", "INFINI", "WALL")] == [10, 2, 2]
    # heat-conduction boundaries: ghost cells at the face centres, zero volume
    b = np.arange(md.nface_int, md.nface)
    assert np.array_equal(md.cell_centre[md.fc2[b]], md.face_centre[b])
    assert np.all(md.cell_volume[md.fc2[b]] == 0.0)


@pytest.mark.parametrize("name,ncell,fams", [
    ("square-quad10.cgns", 100, {"LEFT-DOWN": 5, "RIGHT": 10, "TOP": 10, "BOTTOM": 10, "LEFT-UP": 5}),
    ("rect4x1.cgns", 200, {"LEFT": 10, "RIGHT": 10, "UP": 20, "DOWN": 20}),
])
def test_reads_face_bc_meshes_as_the_oracle_builds_them(golden_dir, name, ncell, fams):
    raw = cgns.read_cgns(golden_dir / name)
    assert all(len(m) == 2 for m in raw.marks)            # FaceCenter tags: face element numbers
    bcs = [(f, umesh.BC_SYMMETRY, "", (0, 0, 0)) for f in fams]
    md = ty.preprocess(raw, 2, bcs)
    assert md.ncell_int == ncell
    assert {f: len(md.faces_of(f)) for f in fams} == fams
    om = op.Mesh.from_raw(raw).build(2, bcs)
    ex = om.export()
    assert np.array_equal(ex["fc1"], md.fc1) and np.array_equal(ex["fc2"], md.fc2)
    for a, b in (("fcentre", "face_centre"), ("fnormal", "face_normal"), ("ccentre", "cell_centre"),
                 ("cvol", "cell_volume"), ("fsurf", "face_surface")):
        assert np.array_equal(ex[a], getattr(md, b)), a


def test_rejects_non_adf(tmp_path):
    p = tmp_path / "x.cgns"
    p.write_bytes(b"HDF5 is not ADF" + bytes(300))
    with pytest.raises(cgns.CgnsError):
        cgns.read_cgns(p)


def tube_kdif(golden_dir):
    raw = cgns.read_cgns(golden_dir / "tube.cgns")
    md = ty.preprocess(raw, 2, TUBE_BCS)
    om = op.Mesh.from_raw(raw).build(2, TUBE_BCS)
    kind = np.zeros(md.nface, np.int32)
    value = np.zeros(md.nface)
    kind[md.faces_of("SYM")] = op.KBC_EXTRAPOLATE             # TYPE = EXTRAPOLATE, ORDER = QUANTITY
    kind[md.faces_of("INFINI")], value[md.faces_of("INFINI")] = op.KBC_ISOTHERMAL, 2000.0
    kind[md.faces_of("WALL")], value[md.faces_of("WALL")] = op.KBC_ISOTHERMAL, 1000.0
    return md, om, kind, value


def read_monres(path):
    return np.loadtxt(path)[:, 1]


def read_probe(path):
    return [ln.split()[2] for ln in open(path) if ln.strip()]


@pytest.mark.parametrize("inversion,max_it", [("CGS", 10), ("BICG", 10), ("GMRES", 50)])
def test_oracle_reproduces_isoth(golden_dir, inversion, max_it):
    """NRG/KDIF/ISOTH-{CGS,BICG,GMRES}: tube.cgns, CONDUCT 10, HEATCAPA 1, FOURIER 20, IMPLICIT
    with Typhon's dlu_cgs, dlu_bicg or dlu_gmres (NKRYLOV 10) at their default IMP_MAX_IT and
    INV_RES 1e-4, DISSIPATIVE_FLUX FULL, T0 100, walls at 1000 and 2000, RESIDUALS 0.1 per
    cycle and 1e-5 overall."""
    md, om, kind, value = tube_kdif(golden_dir)
    k = op.Kdif(om, op.KDIF_FULL, 1.0, np.full(om.ncell_int, 10.0), kind, value)
    k.set_T(np.full(om.ncell, 100.0))
    lr, avg, end = k.typhon_steady(20.0, 10.0, cycle_res=0.1, global_res=1e-5, cgs_maxres=1e-4, cgs_max_it=max_it,
                                   inversion=inversion, nkrylov=10)
    gold = read_monres(golden_dir / f"KDIF-ISOTH-{inversion}__monres.001")
    assert len(lr) == len(gold) == 929
    assert np.abs(lr - gold).max() < 1e-10
    assert list(end) == [125, 326, 527, 728, 929]
    # Typhon prints 0.dddddddd E+xx: eight significant digits
    assert ["%.7E" % a for a in avg] == ["%.7E" % float(v) for v in
                                         read_probe(golden_dir / f"KDIF-ISOTH-{inversion}__Average_T.tmon")]
