"""Rotational periodicity (BLOCK:PERIODICITY TYPE = ROTATION): Typhon's NRG/MESH/CON/PER2D-ROT.

A 30-degree sector of an annulus (perrot2d.cgns, 2582 triangles), RIGHT connected to LEFT by a
rotation of 30 degrees about z, symmetry on RMIN and RMAX; HLLC + MUSCL + van Albada, forward
Euler (the default METHOD) at CFL 0.6, 20 cycles of 5e-4 s from a pressure ring
P = 1e5 (1 + 3 exp(-|x^2 + y^2 - 10|)), T = 300 K, at rest.  Typhon writes, per cycle, the
S-weighted average of the ghost primitive states of RMIN and RMAX (histovarNS_RMIN/RMAX,
integ_ustboco.f90:76-100, format e14.6).

What pins the implementation:
* the native preprocessing (GPU side) builds the same mesh, partners and face rotations as the
  oracle;
* a sector with rotational periodicity gives, to rounding, the solution of the full annulus
  tiled from 12 rotated copies of it (no periodicity at all), for the rotation-invariant
  schemes (first order; MUSCL without limiter: LSQ gradients and HLLC are equivariant);
* against Typhon's own output: density and pressure of the first cycle agree to the last
  printed digit.  The mean velocities at RMIN and RMAX (a few 1e-3 m/s, where the flow is
  almost radial) differ by 0.2 % to 11 % from Typhon's, and the runs separate over the
  following cycles; the test records that deviation rather than hiding it.
GPU runs of the same case are in tests/test_gpu_rotational.py.
"""
import numpy as np
import pytest

import oracle_py as op
from flux_props import exact_sector, tiled_annulus

ROT = {"RIGHT": ((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 30.0)}
BCS = [("RIGHT", op.BC_PERIODIC, "LEFT", (0.0, 0.0, 0.0)), ("RMIN", op.BC_SYMMETRY, "", (0.0, 0.0, 0.0)),
       ("RMAX", op.BC_SYMMETRY, "", (0.0, 0.0, 0.0))]
RGAS = 287.14


def initial_prim(cc):
    x, y = cc[:, 0], cc[:, 1]
    p = 1e5 * (1 + 3 * np.exp(-np.abs(x * x + y * y - 10.0)))
    n = len(x)
    return np.stack([p / (RGAS * 300.0), p, np.zeros(n), np.zeros(n), np.zeros(n)])


def read_histo(path):
    return np.loadtxt(path, comments="#")


def print_ulp(v):
    """Half a unit of the last of six printed significant digits (e14.6)."""
    a = np.abs(v)
    return np.where(a > 0, 10.0 ** (np.floor(np.log10(np.where(a > 0, a, 1.0))) - 5), 1e-300)


@pytest.fixture(scope="module")
def raw(golden_dir):
    from typhon_gb300 import cgns
    return cgns.read_cgns(golden_dir / "perrot2d.cgns")


def test_native_preprocessing_matches_oracle(raw):
    import typhon_gb300 as ty
    om = op.Mesh.from_raw(raw).build(2, BCS, rotations=ROT)
    md = ty.preprocess(raw, 2, BCS, rotations=ROT)
    d = om.export()
    assert np.array_equal(md.fc1, d["fc1"]) and np.array_equal(md.fc2, d["fc2"])
    assert np.array_equal(md.cell_centre, d["ccentre"]) and np.array_equal(md.cell_volume, d["cvol"])
    part = md.face_partner - 1
    assert np.array_equal(np.where(part >= 0, part, -1), d["face_partner"])
    assert md.face_rotation is not None
    assert np.array_equal(md.face_rotation, om.face_rotation())
    # the rotation of a RIGHT face is the inverse of its LEFT partner's
    b = np.where(part >= 0)[0]
    R, Rp = md.face_rotation[b], md.face_rotation[part[b]]
    assert np.allclose(np.einsum("fij,fjk->fik", R, Rp), np.eye(3)[None], atol=1e-15)
    assert not np.allclose(R, np.eye(3)[None])


def run_cycles(s, fam_faces, d, ncycle, cycle_dt=0.01 / 20):
    """Typhon's cycle loop (integration_cyclezone.f90:80-170: the last step of a cycle is cut to
    end it) and the S-weighted average of the ghost primitive states of each family per cycle."""
    out = {k: [] for k in fam_faces}
    for _ in range(ncycle):
        t = 0.0
        while True:
            dt = min(s.timestep(), cycle_dt - t)
            end = dt >= cycle_dt - t
            if end:
                dt = cycle_dt - t
            s.rk_step(dt)
            t = t + dt
            if end:
                break
        q = s.get("prim")
        for name, faces in fam_faces.items():
            S = d["fsurf"][faces]
            out[name].append((q[:, d["fc2"][faces]] * S).sum(axis=1) / S.sum())
    return {k: np.array(v) for k, v in out.items()}


def test_oracle_against_per2d_rot_golden(raw, golden_dir):
    """Density and pressure of the first cycle at every printed digit; velocities reported."""
    import typhon_gb300 as ty
    om = op.Mesh.from_raw(raw).build(2, BCS, rotations=ROT)
    d = om.export()
    s = op.Solver(om, op.SCH_HLLC, op.HRES_MUSCL, op.LIM_ALBADA, op.POSTLIM_NONE, op.GRAD_LSQ, rk="EXPLICIT",
                  cfl=0.6, rgas=RGAS)
    s.set_prim(initial_prim(d["ccentre"]))
    md = ty.preprocess(raw, 2, BCS, rotations=ROT)
    out = run_cycles(s, {k: md.faces_of(k) for k in ("RMIN", "RMAX")}, d, 3)
    for name, val in out.items():
        gold = read_histo(golden_dir / f"PER2D-ROT__histovarNS_{name}")
        assert gold.shape == (20, 6)
        err = np.abs(val[0, :2] - gold[0, 1:3]) / (0.5 * print_ulp(gold[0, 1:3]))
        assert err.max() <= 1.0 + 1e-6, (name, val[0, :2], gold[0, 1:3])
        # density and pressure stay within a few printed units over three cycles
        rel = np.abs(val[:, :2] - gold[:3, 1:3]) / gold[:3, 1:3]
        assert rel.max() < 2e-5, (name, rel.max())
        # the mean velocities: same direction and magnitude to ~10 % (the known deviation)
        uv, ug = val[:, 2:4], gold[:3, 3:5]
        cosang = (uv * ug).sum(axis=1) / np.linalg.norm(uv, axis=1) / np.linalg.norm(ug, axis=1)
        assert cosang.min() > 0.99, (name, cosang)
        ratio = np.linalg.norm(uv, axis=1) / np.linalg.norm(ug, axis=1)
        assert np.all(np.abs(ratio - 1) < 0.1), (name, ratio)


@pytest.fixture(scope="module")
def sector_and_annulus(raw):
    sector = exact_sector(raw)
    ring = tiled_annulus(sector)
    bring = [("RMIN", op.BC_SYMMETRY, "", (0.0, 0.0, 0.0)), ("RMAX", op.BC_SYMMETRY, "", (0.0, 0.0, 0.0))]
    ms = op.Mesh.from_raw(sector).build(2, BCS, rotations=ROT)
    ma = op.Mesh.from_raw(ring).build(2, bring)
    return ms, ma


@pytest.mark.parametrize("hres", ["NONE", "MUSCL"])
def test_sector_equals_full_annulus(sector_and_annulus, hres):
    ms, ma = sector_and_annulus
    ds, da = ms.export(), ma.export()
    nc = ms.ncell_int
    assert ma.ncell_int == 12 * nc
    # copy 0 of the ring is the sector itself, cell by cell
    assert np.allclose(da["ccentre"][:nc], ds["ccentre"][:nc], rtol=0, atol=1e-12)
    assert np.allclose(da["cvol"][:nc], ds["cvol"][:nc], rtol=1e-12, atol=0)
    kw = dict(highres=op.HRES_MUSCL if hres == "MUSCL" else op.HRES_NONE,
              limiter=op.LIM_NONE, gradmeth=op.GRAD_LSQ if hres == "MUSCL" else op.GRAD_NONE,
              rk="RK2", cfl=0.6, rgas=RGAS)
    ss = op.Solver(ms, op.SCH_HLLC, **kw)
    sa = op.Solver(ma, op.SCH_HLLC, **kw)
    ss.set_prim(initial_prim(ds["ccentre"]))
    sa.set_prim(initial_prim(da["ccentre"]))
    dt = 0.5 * min(ss.timestep(), sa.timestep())
    for _ in range(40):
        ss.rk_step(dt)
        sa.rk_step(dt)
    qs, qa = ss.get("prim")[:, :nc], sa.get("prim")
    speed = np.abs(qs[2:4]).max()
    assert speed > 1.0                                   # the ring has started to move
    assert np.abs(qs[:2] - qa[:2, :nc]).max() / np.abs(qs[:2]).max() < 1e-12
    assert np.abs(qs[2:4] - qa[2:4, :nc]).max() / speed < 1e-10
    # the ring's other copies are the rotated sector
    for k in (1, 5, 11):
        t = np.radians(30.0 * k)
        R = np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]])
        uk = R @ qs[2:4]
        assert np.abs(uk - qa[2:4, k * nc:(k + 1) * nc]).max() / speed < 1e-9
