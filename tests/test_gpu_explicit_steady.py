"""Typhon's steady explicit MUSCL runs on the GPU (expansion-10.cgns, NRG/NS/NUM/HRES/MUSCL).

Grid.ns_steady(method="EXPLICIT") runs the forward-Euler steady driver through
ty_steady_iteration: the residual history equals Typhon's monres.001 at every iteration
(1e-10 in log10) and stops at the same iteration, and the state stays bit-identical to the
oracle's in exact mode (within 1e-12 in fast mode).  From the final state Grid.write_vtk
writes Typhon's typhonNS.vtk byte for byte and Grid.probe gives the MINP / MAXV / VCOMP
probes of AUSM-MUSCLUNS as printed; NS/NUM/FLUX/HLLE's outlet flux and ghost-state histories
come out as printed (its histovar file, of a first-order run, reports ghost conservative
states that accumulate the raw boundary fluxes: ty_ghost_state_set keeps them).  The AUSM-M flux has no Jacobian in Typhon: an implicit step with it
is refused.
"""
import numpy as np
import pytest

import oracle_py as op
from test_explicit_steady_golden import BCS, CASES, GAMMA, HLLE_BCS, RGAS, init_state, oracle_case, read_histo

pytestmark = pytest.mark.gpu

NAMES = {op.SCH_HLLC: "HLLC", op.SCH_AUSMM: "AUSMM"}
HRES = {op.HRES_MUSCL: "MUSCL", op.HRES_MUSCLFAST: "MUSCL-FAST", op.HRES_MUSCLUNS: "MUSCL-UNS"}
LIM = {op.LIM_VLEER: "VANLEER", op.LIM_ALBADA: "ALBADA"}


@pytest.fixture(scope="module")
def ty():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from typhon_gb300 import build
    build.build()
    import typhon_gb300
    return typhon_gb300


def gpu_case(ty, golden_dir, name, mode):
    from typhon_gb300 import cgns
    raw = cgns.read_cgns(golden_dir / "expansion-10.cgns")
    md = ty.preprocess(raw, 2, [(f, k, "", (0.0, 0.0, 0.0)) for f, k, _ in BCS])
    sch, hres, lim, res = CASES[name]
    g = ty.Grid(md)
    g.set_spat(NAMES[sch], HRES.get(hres, "NONE"), LIM[lim], gradmeth="LSQ" if hres else "NONE", mode=mode,
               gamma=GAMMA, rgas=RGAS)
    g.set_boundary_params({f: d for f, _, d in BCS if d})
    rho, p, u = init_state(1e5, 300.0, 2.0)
    prim = np.zeros((5, md.ncell))
    prim[0], prim[1], prim[2] = rho, p, u
    g.set_prim(prim)
    out = g.ns_steady(1.0, 1.0, cycle_res=res, global_res=res, method="EXPLICIT", max_iters=20000)
    return raw, md, g, out


@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("name,niter", [("HLLC-MUSCL", 152), ("AUSM-MUSCLFAST", 159), ("HLLC-MUSCLUNS", 227),
                                        ("HLLC-MPI", 174)])
def test_gpu_reproduces_monres(ty, golden_dir, name, niter, mode):
    raw, md, g, out = gpu_case(ty, golden_dir, name, mode)
    gold = np.loadtxt(golden_dir / f"{name}__monres.001")
    assert len(out["log_res"]) == niter and list(out["cycle_end"]) == [niter]
    assert np.abs(out["log_res"] - gold[:, 1]).max() < 1e-10
    _, om, s, _, _ = oracle_case(golden_dir, name)
    U, Uo = g.get_cons(), s.get("cons")[:, :md.ncell_int]
    if mode == "exact":
        assert np.array_equal(U, Uo)
    else:
        for v in range(5):
            assert np.abs(U[v] - Uo[v]).max() <= 1e-12 * np.abs(Uo[v]).max(), v
    g.close()


@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("binary", [False, True])
def test_gpu_vtk_output(ty, golden_dir, tmp_path, mode, binary):
    raw, md, g, out = gpu_case(ty, golden_dir, "AUSM-MUSCLFAST", mode)
    path = tmp_path / "typhonNS.vtk"
    g.write_vtk(path, raw, binary=binary)
    if not binary:
        assert path.read_bytes() == (golden_dir / "AUSM-MUSCLFAST__typhonNS.vtk").read_bytes()
    else:
        from typhon_gb300 import vtk
        ref = tmp_path / "ref.vtk"
        q = g.get_prim()
        vtk.write_vtk(ref, raw, scalars=[("RHO", q[0]), ("PS", q[1])], vectors=[("V", q[2:5])], binary=True)
        assert path.read_bytes() == ref.read_bytes()
    g.close()


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_gpu_probes(ty, golden_dir, mode):
    raw, md, g, out = gpu_case(ty, golden_dir, "AUSM-MUSCLUNS", mode)
    assert list(out["cycle_end"]) == [461]
    for name, kind, expr in (("MINP", "VOL_MIN", "sqrt(PS)"), ("MAXV", "VOL_MAX", "V"),
                             ("VCOMP", "VOL_AVERAGE", "V_Y-V_X")):
        gold = float(open(golden_dir / f"AUSM-MUSCLUNS__{name}.tmon").read().split()[2])
        assert "%.7E" % g.probe(kind, expr) == "%.7E" % gold, name
    g.close()


def test_ausmm_has_no_implicit_step(ty, golden_dir):
    raw, md, g, out = gpu_case(ty, golden_dir, "HLLC-MUSCL", "exact")
    g.set_spat("AUSMM", "MUSCL-FAST", "ALBADA", gradmeth="LSQ", gamma=GAMMA, rgas=RGAS)
    with pytest.raises(ty.TyphonError):
        g.implicit_step(1.0, "GMRES")
    g.close()


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_gpu_hlle_histories(ty, golden_dir, mode):
    from typhon_gb300 import cgns
    raw = cgns.read_cgns(golden_dir / "square-quad10.cgns")
    md = ty.preprocess(raw, 2, [(f, k, "", (0.0, 0.0, 0.0)) for f, k, _ in HLLE_BCS])
    g = ty.Grid(md)
    g.set_spat("HLLE", mode=mode, gamma=GAMMA, rgas=RGAS)
    g.set_boundary_params({f: d for f, _, d in HLLE_BCS if d})
    rho, p, u = init_state(1e5, 300.0, 2.0)
    prim = np.zeros((5, md.ncell))
    prim[0], prim[1], prim[2] = rho, p, u
    g.set_prim(prim)
    g.set_ghost_prim(prim[:, md.ncell_int:])   # Typhon initialises its ghost cells with the state
    out = g.ns_steady(1.0, 1.0, cycle_res=0.3, global_res=1e-4, method="EXPLICIT", history="RIGHT")
    gf = read_histo(golden_dir / "HLLE-EXPLICIT__histofluxNS_RIGHT")
    gv = read_histo(golden_dir / "HLLE-EXPLICIT__histovarNS_RIGHT")
    assert len(out["cycle_end"]) == 8 and len(gv) == 8
    for c in range(8):
        assert ["%.5E" % v for v in out["flux"][c]] == ["%.5E" % v for v in gf[c]], c
        # the ghost rows' conservative states, as Typhon's first-order run keeps them
        assert ["%.5E" % v for v in out["ghost"][c]] == ["%.5E" % v for v in gv[c]], c
    g.close()


def test_gpu_ghost_rows_match_oracle_bitwise(ty, golden_dir):
    """Exact mode: the ghost conservative bookkeeping reproduces the oracle's ghost primitive
    states bit for bit after RK3-SSP steps (every row of Typhon's Runge-Kutta combination);
    a box with symmetry planes and a far field, first-order HLLC (inlets and outlets call pow,
    whose last bit may differ between CUDA and the C library)."""
    raw = ty.read_tym(golden_dir / "quad20x10.tym")
    bcs = [("IMIN", op.BC_FARFIELD, "", (0.0, 0.0, 0.0)), ("IMAX", op.BC_FARFIELD, "", (0.0, 0.0, 0.0)),
           ("JMIN", op.BC_SYMMETRY, "", (0.0, 0.0, 0.0)), ("JMAX", op.BC_SYMMETRY, "", (0.0, 0.0, 0.0))]
    md = ty.preprocess(raw, 2, bcs)
    om = op.Mesh.from_tym(golden_dir / "quad20x10.tym").build(2, bcs)
    free = (1.0, 1.0 / 1.4, 0.5, 0.1, 0.0)
    g = ty.Grid(md)
    g.set_spat("HLLC", mode="exact", farfield=free)
    c = md.cell_centre
    n = md.ncell
    prim = np.stack([1.0 + 0.1 * np.exp(-((c[:, 0] - 1.0) ** 2 + (c[:, 1] - 0.5) ** 2) / 0.02), np.full(n, 1 / 1.4),
                     np.full(n, 0.5), 0.1 + 0.05 * np.sin(3.0 * c[:, 0]), np.zeros(n)])
    g.set_prim(prim)
    g.set_ghost_prim(prim[:, md.ncell_int:])
    s = op.Solver(om, op.SCH_HLLC, rk="RK3-SSP", farfield=free)
    s.set_prim(prim)
    for _ in range(4):
        dt = s.timestep()
        g.treelevel_rungekutta("RK3-SSP", dt)
        s.rk_step(dt)
    nci = md.ncell_int
    assert np.array_equal(g.get_cons(), s.get("cons")[:, :nci])
    assert np.array_equal(g.ghost_prim(), s.get("prim")[:, nci:])
    g.close()


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_gpu_local_time_step_matches_oracle(ty, golden_dir, mode):
    """DTCALC = LOCAL_STABILITY_CONDITION: the same iterations as the oracle, and in exact mode
    the same state bit for bit."""
    from typhon_gb300 import cgns
    raw = cgns.read_cgns(golden_dir / "expansion-10.cgns")
    md = ty.preprocess(raw, 2, [(f, k, "", (0.0, 0.0, 0.0)) for f, k, _ in BCS])
    g = ty.Grid(md)
    g.set_spat("HLLC", "MUSCL", "VANLEER", gradmeth="LSQ", mode=mode, gamma=GAMMA, rgas=RGAS)
    g.set_boundary_params({f: d for f, _, d in BCS if d})
    rho, p, u = init_state(1e5, 300.0, 2.0)
    prim = np.zeros((5, md.ncell))
    prim[0], prim[1], prim[2] = rho, p, u
    g.set_prim(prim)
    out = g.ns_steady(1.0, 1.0, cycle_res=1e-2, global_res=1e-2, method="EXPLICIT", local_dt=True)
    om = op.Mesh.from_raw(raw).build(2, [(f, k, "", (0.0,) * 3, (0.0,) * 3, d) if d else (f, k, "", (0.0,) * 3)
                                          for f, k, d in BCS])
    s = op.Solver(om, op.SCH_HLLC, highres=op.HRES_MUSCL, limiter=op.LIM_VLEER, gradmeth=op.GRAD_LSQ, gamma=GAMMA,
                  rgas=RGAS, rk="EXPLICIT")
    s.set_prim(prim)
    lr, _, _, end = s.typhon_steady(1.0, 1.0, cycle_res=1e-2, global_res=1e-2, method="EXPLICIT", local_dt=True)
    assert list(out["cycle_end"]) == list(end)
    assert np.abs(out["log_res"] - lr).max() < 1e-10
    U, Uo = g.get_cons(), s.get("cons")[:, :md.ncell_int]
    if mode == "exact":
        assert np.array_equal(U, Uo)
    else:
        for v in range(5):
            assert np.abs(U[v] - Uo[v]).max() <= 1e-12 * np.abs(Uo[v]).max(), v
    g.close()
