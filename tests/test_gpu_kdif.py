"""GPU heat conduction (KDIF) against the oracle, through the C ABI.

Exact mode: ghost temperatures, gradients, face fluxes, Jacobians, the symmetrised
implicit matrix and its mat-vec are bit for bit the oracle's; the conjugate-gradient
update agrees with the oracle's to the solve tolerance.  The FP32 conjugate gradients
inside FP64 iterative refinement reach a 1e-12 relative residual and the FP64 solution.
"""
import numpy as np
import pytest

import oracle_py as op

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ty():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from typhon_gb300 import build
    build.build()
    import typhon_gb300
    return typhon_gb300


def box_case(ty, n=6, jitter=0.1, seed=5):
    from typhon_gb300 import umesh
    raw = umesh.gen_tet_box(n, 1.0, jitter=jitter, seed=seed)
    bcs = [(f, umesh.BC_WALL, "", (0, 0, 0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX", "KMIN", "KMAX")]
    md = ty.preprocess(raw, 3, bcs)
    om = op.Mesh.from_raw(raw).build(3, bcs)
    fc = md.face_centre
    kind = np.zeros(md.nface, np.int32)
    val = np.zeros(md.nface)
    for f in range(md.nface_int, md.nface):
        if abs(fc[f, 0]) < 1e-12:
            kind[f], val[f] = op.KBC_ISOTHERMAL, 0.0
        elif abs(fc[f, 0] - 1.0) < 1e-12:
            kind[f], val[f] = op.KBC_ISOTHERMAL, 1.0
        elif abs(fc[f, 1]) < 1e-12:
            kind[f], val[f] = op.KBC_FLUX, 0.25
        elif abs(fc[f, 1] - 1.0) < 1e-12:
            kind[f], val[f] = op.KBC_EXTRAPOLATE, 0.0
        else:
            kind[f], val[f] = op.KBC_FLUX, 0.0
    rng = np.random.default_rng(seed)
    kc = np.exp(0.5 * rng.standard_normal(md.ncell_int))
    T0 = rng.uniform(0.2, 0.8, md.ncell)
    return md, om, kind, val, kc, T0


@pytest.mark.parametrize("scheme", ["COMPACT", "CELL-AVERAGE", "FULL"])
def test_exact_kdif_bitwise(ty, scheme):
    md, om, kind, val, kc, T0 = box_case(ty)
    osch = {"COMPACT": op.KDIF_COMPACT, "CELL-AVERAGE": op.KDIF_CELLAVG, "FULL": op.KDIF_FULL}[scheme]
    g = ty.Grid(md)
    g.set_spat("HLLC", mode="exact")
    g.kdif_setup(kc, kind, val, flux=scheme, heat_capacity=1.7)
    g.kdif_set_temperature(T0)
    k = op.Kdif(om, osch, 1.7, kc, kind, val)
    k.set_T(T0)
    dt = 2e-3
    R = g.kdif_residual(dt)
    k.rhs(dt)
    nci = md.ncell_int
    assert np.array_equal(g.kdif_get("T"), k.get("T")), "ghost temperatures"
    if scheme != "COMPACT":
        assert np.array_equal(g.kdif_get("grad"), k.get("grad")[:, :nci]), "gradient"
    assert np.array_equal(g.kdif_get("flux"), k.get("flux")), "face flux"
    assert np.array_equal(g.kdif_get("jac"), k.get("jac")), "Jacobian"
    assert np.array_equal(g.kdif_get("balance"), k.get("balance")), "balance"
    assert np.array_equal(R, k.get("residu")[:nci]), "residual"
    st = g.kdif_implicit_step(dt, "CG", tol=1e-13)
    it, rel = k.implicit_step(dt, tol=1e-13)
    assert np.array_equal(g.kdif_get("diag"), k.get("diag")), "diagonal"
    x = np.random.default_rng(1).standard_normal(nci)
    assert np.array_equal(g.kdif_matvec(x), k.matvec(x)), "mat-vec"
    assert st["rel_res"] < 1e-13
    dT, dTo = g.kdif_temperature() - T0[:nci], k.get("T")[:nci] - T0[:nci]
    assert np.linalg.norm(dT - dTo) / np.linalg.norm(dTo) < 1e-11


@pytest.mark.parametrize("solver", ["CG32", "CG-MIXED"])
def test_mixed_precision_solvers_reach_fp64(ty, solver):
    """FP32 CG inside FP64 refinement, and CG on FP32 face conductances restarted on the FP64
    matrix at 1e-6: both reach the FP64 CG solution, to 1e-12 on the FP64 system."""
    md, om, kind, val, kc, T0 = box_case(ty, n=8)
    kc = kc * np.exp(np.random.default_rng(3).standard_normal(kc.shape))   # heterogeneous k
    sols = {}
    for sv in ("CG", solver):
        g = ty.Grid(md)
        g.set_spat("HLLC", mode="fast")
        g.kdif_setup(kc, kind, val, flux="FULL", heat_capacity=1.0)
        g.kdif_set_temperature(T0)
        for _ in range(3):
            st = g.kdif_implicit_step(1e-2, sv, tol=1e-12)
            assert st["rel_res"] < 1e-12, st
            if sv == "CG32":
                assert st["refinements"] >= 2
            if sv == "CG-MIXED":
                assert st["refinements"] == 1     # switched from FP32 to FP64 conductances
        sols[sv] = g.kdif_temperature()
    assert np.linalg.norm(sols[solver] - sols["CG"]) / np.linalg.norm(sols["CG"]) < 1e-11


def test_fast_kdif_close(ty):
    md, om, kind, val, kc, T0 = box_case(ty)
    g = ty.Grid(md)
    g.set_spat("HLLC", mode="fast")
    g.kdif_setup(kc, kind, val, flux="FULL", heat_capacity=1.0)
    g.kdif_set_temperature(T0)
    k = op.Kdif(om, op.KDIF_FULL, 1.0, kc, kind, val)
    k.set_T(T0)
    for _ in range(3):
        g.kdif_implicit_step(5e-3, "CG", tol=1e-13)
        k.implicit_step(5e-3, tol=1e-13)
    T, To = g.kdif_temperature(), k.get("T")[:md.ncell_int]
    assert np.linalg.norm(T - To) / np.linalg.norm(To) < 1e-12


def test_kdif_errors(ty):
    md, om, kind, val, kc, T0 = box_case(ty, n=2)
    g = ty.Grid(md)
    with pytest.raises(ty.TyphonError):
        g.kdif_residual(1e-3)                        # no set-up
    bad = kind.copy()
    bad[md.nface - 1] = 0
    with pytest.raises(ty.TyphonError):
        g.kdif_setup(kc, bad, val)                   # boundary face without a kind
    with pytest.raises(ty.TyphonError):
        g.kdif_setup(-kc, kind, val)                 # non-positive conductivity


def test_typhon_steady_run_reproduces_isoth_cgs(ty, golden_dir, tmp_path):
    """NRG/KDIF/ISOTH-CGS through the GPU: Typhon's steady driver (Grid.kdif_steady) over
    ty_kdif_implicit_step.  The GPU solves each step to 1e-13 where Typhon's CGS stops at
    INV_RES 1e-4: on this 10-cell system both are converged to about 1e-8 in the log10
    residual, which is the tolerance; the cycle structure and the printed averages agree."""
    from typhon_gb300 import cgns, umesh
    raw = cgns.read_cgns(golden_dir / "tube.cgns")
    bcs = [(f, umesh.BC_HEAT, "", (0, 0, 0)) for f in ("SYM", "INFINI", "WALL")]
    md = ty.preprocess(raw, 2, bcs)
    kind = np.zeros(md.nface, np.int32)
    val = np.zeros(md.nface)
    kind[md.faces_of("SYM")] = op.KBC_EXTRAPOLATE
    kind[md.faces_of("INFINI")], val[md.faces_of("INFINI")] = op.KBC_ISOTHERMAL, 2000.0
    kind[md.faces_of("WALL")], val[md.faces_of("WALL")] = op.KBC_ISOTHERMAL, 1000.0
    for mode in ("exact", "fast"):
        g = ty.Grid(md)
        g.set_spat("HLLC", mode=mode)
        g.kdif_setup(np.full(md.ncell_int, 10.0), kind, val, flux="FULL", heat_capacity=1.0)
        g.kdif_set_temperature(np.full(md.ncell_int, 100.0))
        assert g.kdif_fourier_dt(20.0) == pytest.approx(2.0 * 20.0 * 100.0 ** 2 / 850.0 / 10.0, rel=1e-14)
        out = g.kdif_steady(20.0, cycle_res=0.1, global_res=1e-5, tol=1e-13)
        gold = np.loadtxt(golden_dir / "KDIF-ISOTH-CGS__monres.001")[:, 1]
        assert len(out["log_res"]) == len(gold) == 929
        assert np.abs(out["log_res"] - gold).max() < 1e-7
        assert list(out["cycle_end"]) == [125, 326, 527, 728, 929]
        probe = [float(ln.split()[2]) for ln in open(golden_dir / "KDIF-ISOTH-CGS__Average_T.tmon") if ln.strip()]
        assert ["%.7E" % a for a in out["cycle_avg"]] == ["%.7E" % p for p in probe]
        if mode == "exact":
            # VTK output of a heat-conduction zone: the quad cells and the scalar TS
            from typhon_gb300 import vtk
            path = tmp_path / "tube.vtk"
            g.kdif_write_vtk(path, raw)
            f = vtk.read_vtk_ascii(path)
            assert f["types"] == [9] * 10 and len(f["points"]) == 18
            assert np.allclose(f["TS"], g.kdif_temperature(), rtol=1e-8, atol=0)
        g.close()


def test_heat_boundary_mesh_refuses_navier_stokes(ty, golden_dir):
    from typhon_gb300 import cgns, umesh
    raw = cgns.read_cgns(golden_dir / "tube.cgns")
    md = ty.preprocess(raw, 2, [(f, umesh.BC_HEAT, "", (0, 0, 0)) for f in ("SYM", "INFINI", "WALL")])
    g = ty.Grid(md)
    g.set_spat("HLLC", mode="exact")
    prim = np.tile(np.array([[1.0], [1.0], [0.1], [0.0], [0.0]]), (1, md.ncell))
    g.set_prim(prim)
    with pytest.raises(ty.TyphonError):
        g.integration_grid(1e-3)
    g.close()
