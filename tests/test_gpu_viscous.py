"""GPU parity of the laminar viscous flux and the moving adiabatic walls (through the C ABI).

Exact mode reproduces the oracle bit for bit; Typhon's golden VISCOUS CELLAVG / CELLFULL
monitors are replayed through the GPU; fast mode stays within 1e-12 relative L2 per
conserved variable.
"""
import numpy as np
import pytest

import oracle_py as op

pytestmark = pytest.mark.gpu

FAST_RTOL = 1e-12
MXLAY_BCS = [("IMIN", op.BC_PERIODIC, "IMAX", (1.0, 0.0, 0.0)),
             ("JMIN", op.BC_WALL, "", (0.0, 0.0, 0.0), (-1.0, 0.0, 0.0)),
             ("JMAX", op.BC_WALL, "", (0.0, 0.0, 0.0), (1.0, 0.0, 0.0))]
VISC = {"CELL-AVERAGE": op.VISC_CELLAVG, "FULL": op.VISC_CELLFULL}


@pytest.fixture(scope="module")
def ty():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from typhon_gb300 import build
    build.build()
    import typhon_gb300
    return typhon_gb300


def mxlay(ty, golden_dir):
    md = ty.preprocess(ty.read_tym(golden_dir / "mxlay2x20quad-h50.tym"), 2, MXLAY_BCS)
    om = op.Mesh.from_tym(golden_dir / "mxlay2x20quad-h50.tym").build(2, MXLAY_BCS)
    from scipy.special import erf
    y = md.cell_centre[:, 1]
    n = md.ncell
    prim = np.stack([np.ones(n), np.full(n, 100 / 1.4), erf(y / 2 / np.sqrt(1.0)), np.zeros(n), np.zeros(n)])
    return md, om, prim


def relerr(a, b):
    """Relative L2 error per conserved variable of Typhon's field: rho, rhoE and the momentum
    vector rho u (the field holds two scalars and one vector, and update_field.f90:54-60
    measures the vector by its norm, so a momentum component that is near zero is measured
    against the momentum, not against itself)."""
    d = a - b
    num = [np.linalg.norm(d[0]), np.linalg.norm(d[1]), np.linalg.norm(d[2:5])]
    den = [np.linalg.norm(b[0]), np.linalg.norm(b[1]), np.linalg.norm(b[2:5])]
    return np.array(num) / np.maximum(np.array(den), 1e-300)


@pytest.mark.parametrize("dflux", ["CELL-AVERAGE", "FULL"])
@pytest.mark.parametrize("scheme,highres,limiter", [("HLLC", "MUSCL-FAST", "ALBADA"), ("ROE", "MUSCL-UNS", "NONE"),
                                                    ("RUSANOV", "NONE", "NONE")])
def test_exact_viscous_residual_bitwise(ty, golden_dir, dflux, scheme, highres, limiter):
    md, om, prim = mxlay(ty, golden_dir)
    g = ty.Grid(md)
    g.set_spat(scheme, highres, limiter, mode="exact", dissipative_flux=dflux, kin_visc=1.0)
    g.set_prim(prim)
    sch = {"HLLC": op.SCH_HLLC, "ROE": op.SCH_ROE, "RUSANOV": op.SCH_RUSANOV}[scheme]
    hr = {"MUSCL-FAST": op.HRES_MUSCLFAST, "MUSCL-UNS": op.HRES_MUSCLUNS, "NONE": op.HRES_NONE}[highres]
    lim = {"ALBADA": op.LIM_ALBADA, "NONE": op.LIM_NONE}[limiter]
    s = op.Solver(om, sch, hr, lim, gradmeth=op.GRAD_LSQ, rk="RK25BB", cfl=0.5,
                  viscous=VISC[dflux], visc_kin=1.0)
    s.set_prim(prim)
    dt = s.timestep()
    assert g.calc_zonetimestep(0.5) == dt
    R = g.integration_grid(dt)
    s.rhs(dt)
    assert np.array_equal(g.debug("flux"), s.get("flux")), "face flux"
    assert np.array_equal(R, s.get("residu")[:, :md.ncell_int]), "residual"
    for _ in range(2):
        dt = s.timestep()
        g.treelevel_rungekutta("RK25BB", dt)
        s.rk_step(dt)
    assert np.array_equal(g.get_cons(), s.get("cons")[:, :md.ncell_int])


def _print_ulp(v):
    return 10.0 ** (np.floor(np.log10(np.abs(v))) - 7)


@pytest.mark.parametrize("name,dflux", [("CELLAVG", "CELL-AVERAGE"), ("CELLFULL", "FULL")])
def test_nrg_viscous_replayed_on_gpu(ty, golden_dir, name, dflux):
    """NRG/NS/NUM/FLUX/VISCOUS/<name> through the GPU (exact mode): VXERR and DELTA."""
    from scipy.special import erf
    md, om, prim = mxlay(ty, golden_dir)
    g = ty.Grid(md)
    g.set_spat("HLLC", "MUSCL-FAST", "ALBADA", mode="exact", dissipative_flux=dflux, kin_visc=1.0)
    g.set_prim(prim)
    nci = md.ncell_int
    vol = md.cell_volume[:nci]
    y = md.cell_centre[:nci, 1]
    vxerr, delta, t = [], [], 0.0
    for _ in range(10):
        g.integration_cyclezone("RK25BB", 0.5, 1.0)
        t = t + 1.0
        vx = g.get_prim()[2]
        vxerr.append(np.sum((vx - erf(y / 2 / np.sqrt(t + 1.0))) ** 2 * vol) / np.sum(vol))
        delta.append(np.sum(2 * 50 * (1 - vx * vx) * vol) / np.sum(vol))
    for out, f in ((vxerr, "VXERR"), (delta, "DELTA")):
        gold = np.loadtxt(golden_dir / f"VISCOUS-{name}-{f}__{f}.tmon")[:, 2]
        err = np.abs(np.array(out) - gold) / _print_ulp(gold)
        assert err.max() <= 0.5 + 1e-3, (f, err.max())


@pytest.mark.parametrize("dflux", ["CELL-AVERAGE", "FULL"])
def test_fast_viscous_close(ty, golden_dir, dflux):
    md, om, prim = mxlay(ty, golden_dir)
    g = ty.Grid(md)
    g.set_spat("HLLC", "MUSCL", "ALBADA", mode="fast", dissipative_flux=dflux, kin_visc=1.0)
    g.set_prim(prim)
    s = op.Solver(om, op.SCH_HLLC, op.HRES_MUSCL, op.LIM_ALBADA, gradmeth=op.GRAD_LSQ, rk="RK25BB", cfl=0.5,
                  viscous=VISC[dflux], visc_kin=1.0)
    s.set_prim(prim)
    for _ in range(5):
        dt = s.timestep()
        g.treelevel_rungekutta("RK25BB", dt)
        s.rk_step(dt)
    rel = relerr(g.get_cons(), s.get("cons")[:, :md.ncell_int])
    assert np.all(rel <= FAST_RTOL), rel


def test_sutherland_tgv_fast_close(ty):
    """3D laminar Navier-Stokes with Sutherland viscosity on the periodic tet box, fast mode."""
    from typhon_gb300 import cases
    L = 2 * np.pi
    raw = ty.gen_tet_box(6, L, jitter=0.05, seed=1234)
    bcs = ty.periodic_box_bcs((L, L, L))
    md = ty.preprocess(raw, 3, bcs)
    om = op.Mesh.from_raw(raw).build(3, bcs)
    prim = cases.taylor_green(md.cell_centre)
    prim[1] *= 287.14 * 300.0 / prim[1].mean() * prim[0].mean()   # air-like temperature ~300 K
    g = ty.Grid(md)
    g.set_spat("ROE", "MUSCL-UNS", "NONE", "BARTH", mode="fast", dissipative_flux="FULL", viscosity="SUTHERLAND")
    g.set_prim(prim)
    s = op.Solver(om, op.SCH_ROE, op.HRES_MUSCLUNS, op.LIM_NONE, op.POSTLIM_BARTH, op.GRAD_LSQ, rk="RK3-SSP",
                  cfl=0.8, viscous=op.VISC_CELLFULL, visc_law=1)
    s.set_prim(prim)
    for _ in range(3):
        dt = s.timestep()
        g.treelevel_rungekutta("RK3-SSP", dt)
        s.rk_step(dt)
    rel = relerr(g.get_cons(), s.get("cons")[:, :md.ncell_int])
    assert np.all(rel <= FAST_RTOL), rel
