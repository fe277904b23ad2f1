"""Pin the CPU oracle against Typhon's own non-regression golden files.

Typhon writes monitors with format (i5,2e16.8) (SOURCE/MAIN/write_monitors_cycle.f90:67):
every value must agree to within half a unit of its last printed digit.
"""
import numpy as np
import pytest

import oracle_py as op

RK_CASES = {  # NRG/TIME/RUNGEKUTTA/<case>/main.rpm: METHOD, CFL
    "RK2": ("RK2", 0.8), "RK2-SSP": ("RK2-SSP", 0.8), "RK3-SSP": ("RK3-SSP", 1.5),
    "RK4": ("RK4", 2.0), "RK25BB": ("RK25BB", 2.5), "RK26BB": ("RK26BB", 2.5),
    # the RK12BS and RK13BS inputs say METHOD = RK25BB
    "RK12BS": ("RK25BB", 2.5), "RK13BS": ("RK25BB", 2.5),
}


def print_ulp(values):
    return 10.0 ** (np.floor(np.log10(np.abs(values))) - 7)


@pytest.fixture(scope="module")
def quad20(golden_dir, oracle):
    return op.Mesh.from_tym(golden_dir / "quad20x20.tym").build(2, op.PERIODIC_UNIT_SQUARE)


@pytest.mark.parametrize("case", list(RK_CASES))
def test_rungekutta_rhoerr(case, quad20, golden_dir):
    method, cfl = RK_CASES[case]
    out, nsteps = op.run_nrg(1, quad20, method, cfl)
    gold = np.loadtxt(golden_dir / f"{case}__RHOERR.tmon")
    assert gold.shape == (100, 3)
    np.testing.assert_allclose(gold[:, 1], 0.001 * np.arange(1, 101), rtol=1e-7)
    err = np.abs(out - gold[:, 2]) / print_ulp(gold[:, 2])
    assert err.max() <= 0.5 + 1e-6, (case, err.max(), int(np.argmax(err)))


def test_per2d_trans_rhodev(quad20, golden_dir):
    out, nsteps = op.run_nrg(2, quad20, "RK3-SSP", 1.0)
    gold = np.loadtxt(golden_dir / "PER2D-TRANS__RHODEV.tmon")
    err = np.abs(out - gold[:, 2]) / print_ulp(gold[:, 2])
    assert err.max() <= 0.5 + 1e-6, err.max()


def test_quad20_mesh_counts(quad20):
    # 20x20 quads: 400 cells, 2*20*21 = 840 faces, 80 periodic boundary faces / ghost cells
    assert (quad20.ncell_int, quad20.nface, quad20.nface_int, quad20.ncell) == (400, 840, 760, 480)
    d = quad20.export()
    assert np.isclose(d["cvol"][:400].sum(), 1.0, rtol=0, atol=1e-14)
    # periodic partners are mutual
    part = d["face_partner"]
    b = np.where(part >= 0)[0]
    assert len(b) == 80 and np.all(part[part[b]] == b)


SYMMETRY_BOX = [(f, op.BC_SYMMETRY, "", (0.0, 0.0, 0.0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX")]


def test_tym_quad_symmetry_pavg(golden_dir, oracle):
    """NRG/MESH/ELEM/TYM-QUAD: HLLC first order, symmetry on all four sides, 10 cycles."""
    m = op.Mesh.from_tym(golden_dir / "quad20x10.tym").build(2, SYMMETRY_BOX)
    out, nsteps = op.run_nrg(3, m, "RK3-SSP", 1.0, ncycle=10, duration=0.005)
    gold = np.loadtxt(golden_dir / "TYM-QUAD__PAVG.tmon")
    err = np.abs(out - gold[:, 2]) / print_ulp(gold[:, 2])
    assert err.max() <= 0.5 + 1e-6, err.max()


MXLAY_BCS = [("IMIN", op.BC_PERIODIC, "IMAX", (1.0, 0.0, 0.0)),
             ("JMIN", op.BC_WALL, "", (0.0, 0.0, 0.0), (-1.0, 0.0, 0.0)),
             ("JMAX", op.BC_WALL, "", (0.0, 0.0, 0.0), (1.0, 0.0, 0.0))]


@pytest.mark.parametrize("which,name", [(4, "CELLAVG"), (5, "CELLFULL")])
def test_viscous_mixing_layer(golden_dir, oracle, which, name):
    """NRG/NS/NUM/FLUX/VISCOUS/<name>: laminar (nu = 1), HLLC + MUSCL-FAST + van Albada,
    periodic in x, adiabatic walls moving at -1 / +1, RK25BB, 10 cycles; monitors VXERR and
    DELTA.  Wall ghost-cell gradients are taken as zero (Typhon never sets them)."""
    m = op.Mesh.from_tym(golden_dir / "mxlay2x20quad-h50.tym").build(2, MXLAY_BCS)
    (vxerr, delta), _ = op.run_nrg(which, m, "RK25BB", 0.5, ncycle=10, duration=10.0)
    for out, f in ((vxerr, "VXERR"), (delta, "DELTA")):
        gold = np.loadtxt(golden_dir / f"VISCOUS-{name}-{f}__{f}.tmon")
        err = np.abs(out - gold[:, 2]) / print_ulp(gold[:, 2])
        assert err.max() <= 0.5 + 1e-6, (f, err.max())
