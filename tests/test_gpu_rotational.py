"""GPU runs with rotational periodicity (Typhon's NRG/MESH/CON/PER2D-ROT sector) against the
oracle, through the C ABI.

Exact mode reproduces the oracle bit for bit: LSQ gradients with the rotated ghost states, face
states rotated from the partner face, residuals, Runge-Kutta states over whole cycles, and the
implicit blocks.  The Typhon history files of the case are replayed on the GPU with the same
bar as the oracle's (density and pressure of the first cycle at every printed digit).
"""
import numpy as np
import pytest

import oracle_py as op
from test_rotational_periodicity import BCS, ROT, RGAS, initial_prim, print_ulp, read_histo

pytestmark = pytest.mark.gpu

OSCH = {"HLLC": op.SCH_HLLC, "ROE": op.SCH_ROE, "RUSANOV": op.SCH_RUSANOV}
OHRES = {"NONE": op.HRES_NONE, "MUSCL": op.HRES_MUSCL, "MUSCL-FAST": op.HRES_MUSCLFAST}
OLIM = {"NONE": op.LIM_NONE, "ALBADA": op.LIM_ALBADA, "MINMOD": op.LIM_MINMOD}


@pytest.fixture(scope="module")
def ty():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from typhon_gb300 import build
    build.build()
    import typhon_gb300
    return typhon_gb300


@pytest.fixture(scope="module")
def sector(ty, golden_dir):
    from typhon_gb300 import cgns
    raw = cgns.read_cgns(golden_dir / "perrot2d.cgns")
    md = ty.preprocess(raw, 2, BCS, rotations=ROT)
    om = op.Mesh.from_raw(raw).build(2, BCS, rotations=ROT)
    assert md.face_rotation is not None
    return md, om


def pair(ty, md, om, scheme, highres, limiter, mode="exact", rk="EXPLICIT", cfl=0.6):
    gm = "NONE" if highres == "NONE" else "LSQ"
    prim = initial_prim(md.cell_centre)
    g = ty.Grid(md)
    g.set_spat(scheme, highres, limiter, gradmeth=gm, mode=mode, rgas=RGAS)
    g.set_prim(prim)
    s = op.Solver(om, OSCH[scheme], OHRES[highres], OLIM[limiter], op.POSTLIM_NONE,
                  op.GRAD_NONE if gm == "NONE" else op.GRAD_LSQ, rk=rk, cfl=cfl, rgas=RGAS)
    s.set_prim(prim)
    return g, s


COMBOS = [("HLLC", "MUSCL", "ALBADA"), ("ROE", "NONE", "NONE"), ("RUSANOV", "MUSCL-FAST", "MINMOD")]


@pytest.mark.parametrize("combo", COMBOS, ids=["-".join(c) for c in COMBOS])
def test_exact_residual_bitwise(ty, sector, combo):
    md, om = sector
    g, s = pair(ty, md, om, *combo)
    dt = s.timestep()
    assert g.calc_zonetimestep(0.6) == dt
    R = g.integration_grid(dt)
    s.rhs(dt)
    nci = md.ncell_int
    if combo[1] != "NONE":
        assert np.array_equal(g.debug("grad")[:, :nci], s.get("grad")[:, :nci]), "gradient"
    assert np.array_equal(g.debug("flux"), s.get("flux")), "face flux"
    assert np.array_equal(R, s.get("residu")[:, :nci]), "residual"


def test_exact_cycles_bitwise(ty, sector):
    md, om = sector
    g, s = pair(ty, md, om, "HLLC", "MUSCL", "ALBADA")
    cycle_dt = 0.01 / 20
    for _ in range(3):
        g.integration_cyclezone("EXPLICIT", 0.6, cycle_dt)
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
    assert np.array_equal(g.get_cons(), s.get("cons")[:, :md.ncell_int])


def test_fast_mode_close(ty, sector):
    md, om = sector
    g, s = pair(ty, md, om, "HLLC", "MUSCL", "ALBADA", mode="fast", rk="RK2")
    for _ in range(5):
        dt = s.timestep()
        g.treelevel_rungekutta("RK2", dt)
        s.rk_step(dt)
    a, b = g.get_cons(), s.get("cons")[:, :md.ncell_int]
    for sl in (slice(0, 1), slice(1, 2), slice(2, 5)):
        assert np.linalg.norm(a[sl] - b[sl]) / np.linalg.norm(b[sl]) < 1e-12


def test_per2d_rot_golden_replayed_on_gpu(ty, sector, golden_dir):
    md, om = sector
    g = ty.Grid(md)
    g.set_spat("HLLC", "MUSCL", "ALBADA", gradmeth="LSQ", mode="exact", rgas=RGAS)
    g.set_prim(initial_prim(md.cell_centre))
    faces = {k: md.faces_of(k) for k in ("RMIN", "RMAX")}
    surf = md.face_surface
    out = {k: [] for k in faces}
    for _ in range(3):
        g.integration_cyclezone("EXPLICIT", 0.6, 0.01 / 20)
        q = g.debug("prim")           # interior and ghost primitive states of the last stage
        for k, f in faces.items():
            ghost = q[:, md.fc2[f]]
            out[k].append((ghost * surf[f]).sum(axis=1) / surf[f].sum())
    for k, v in out.items():
        val = np.array(v)
        gold = read_histo(golden_dir / f"PER2D-ROT__histovarNS_{k}")
        err = np.abs(val[0, :2] - gold[0, 1:3]) / (0.5 * print_ulp(gold[0, 1:3]))
        assert err.max() <= 1.0 + 1e-6, (k, val[0, :2], gold[0, 1:3])
        assert (np.abs(val[:, :2] - gold[:3, 1:3]) / gold[:3, 1:3]).max() < 2e-5


def test_implicit_blocks_bitwise(ty, sector):
    md, om = sector
    g, s = pair(ty, md, om, "HLLC", "MUSCL", "ALBADA", cfl=1.0)
    U0 = g.get_cons()
    st = g.implicit_step(20.0, "GMRES", nkrylov=30, max_it=20, inv_res=1e-10, local_dt=True)
    info, it, l1 = s.implicit_step(20.0, local_dt=True, nkrylov=30, max_it=20, inv_res=1e-10)
    nci, nfi = md.ncell_int, md.nface_int
    for name in ("jacL", "jacR"):
        assert np.array_equal(g.implicit_get(name), s.get_implicit(name)), name
    assert np.array_equal(g.implicit_get("diag"), s.get_implicit("diag")[:nci]), "diag"
    assert np.array_equal(g.implicit_get("rhs"), s.implicit_rhs()[:nci]), "rhs"
    assert st["info"] == info and st["restarts"] == it
    du, du_o = g.get_cons() - U0, s.get("cons")[:, :nci] - U0
    assert np.linalg.norm(du - du_o) / np.linalg.norm(du_o) < 1e-9
