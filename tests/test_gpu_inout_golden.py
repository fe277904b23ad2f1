"""GPU inlets, outlets and the HLLE flux against the oracle, and Typhon's implicit golden run.

* One implicit step on square-quad10.cgns with HLLE, two subsonic inlets, a subsonic outlet
  and symmetry planes, and one on rect4x1.cgns with Rusanov, supersonic inlets and a
  supersonic outlet (its Jacobian folded): the flux Jacobians, blocks, right-hand side and
  the update match the oracle's.  The boundary states use pow, whose CUDA and C library
  results may differ in the last bit, so these comparisons carry a 1e-13 tolerance instead
  of bit equality.
* NRG/TIME/IMPLICIT/GMRES through Grid.ns_steady on the GPU (exact and fast modes): the
  summed outlet fluxes after each of the seven cycles equal Typhon's printed history
  (histofluxNS_RIGHT, six digits).
"""
import numpy as np
import pytest

import oracle_py as op

pytestmark = pytest.mark.gpu

GAMMA, RGAS = 1.4, 287.14
Z3 = (0.0, 0.0, 0.0)


@pytest.fixture(scope="module")
def ty():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from typhon_gb300 import build
    build.build()
    import typhon_gb300
    return typhon_gb300


def init_state(pi, ti, mach):
    g = GAMMA
    gmusd, gsgmu = (g - 1.0) / 2.0, g / (g - 1.0)
    p = pi / (1.0 + gmusd * mach ** 2) ** gsgmu
    rho = p / (RGAS * ti) * (1.0 + gmusd * mach ** 2)
    return rho, p, np.sqrt(g * p / rho) * mach


GMRES_CASE = dict(mesh="square-quad10.cgns", scheme="HLLE", oscheme=op.SCH_HLLE, init=(1e5, 300.0, 2.0),
                  bcs=[("LEFT-UP", op.BC_INLET_SUB, (1.7e5, 200.0, 1.0, 0.0, 0.0)),
                       ("LEFT-DOWN", op.BC_INLET_SUB, (1.2e5, 600.0, 1.0, 0.0, 0.0)),
                       ("RIGHT", op.BC_OUTLET_SUB, (1e5,)),
                       ("TOP", op.BC_SYMMETRY, None), ("BOTTOM", op.BC_SYMMETRY, None)])
SUPERSONIC_CASE = dict(mesh="rect4x1.cgns", scheme="RUSANOV", oscheme=op.SCH_RUSANOV, init=(1e5, 300.0, 4.0),
                       bcs=[("DOWN", op.BC_SYMMETRY, None), ("RIGHT", op.BC_OUTLET_SUP, None),
                            ("LEFT", op.BC_INLET_SUP, (1e5, 300.0, 4.0, 1.0, 0.0, 0.0)),
                            ("UP", op.BC_INLET_SUP, (98497.053, 300.0, 3.60110, 1.0, -0.0967742, 0.0))])


def setup(ty, golden_dir, case, mode="exact", perturb=0.0):
    from typhon_gb300 import cgns
    raw = cgns.read_cgns(golden_dir / case["mesh"])
    gb = [(f, k, "", Z3) for f, k, _ in case["bcs"]]
    ob = [(f, k, "", Z3, Z3, d) if d else (f, k, "", Z3) for f, k, d in case["bcs"]]
    md = ty.preprocess(raw, 2, gb)
    om = op.Mesh.from_raw(raw).build(2, ob)
    rho, p, u = init_state(*case["init"])
    prim = np.zeros((5, md.ncell))
    prim[0], prim[1], prim[2] = rho, p, u
    if perturb:
        x, y = md.cell_centre[:, 0], md.cell_centre[:, 1]
        prim[0] *= 1 + perturb * np.sin(3 * x + 1) * np.cos(2 * y)
        prim[1] *= 1 + perturb * np.cos(2 * x) * np.sin(3 * y + 0.5)
        prim[3] = perturb * u * np.sin(x + 2 * y)
    g = ty.Grid(md)
    g.set_spat(case["scheme"], mode=mode, gamma=GAMMA, rgas=RGAS)
    g.set_boundary_params({f: d for f, _, d in case["bcs"] if d})
    g.set_prim(prim)
    s = op.Solver(om, case["oscheme"], gamma=GAMMA, rgas=RGAS)
    s.set_prim(prim)
    return md, om, g, s


def close(a, b, tol=1e-13):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= tol * scale


@pytest.mark.parametrize("case", [GMRES_CASE, SUPERSONIC_CASE], ids=["subsonic-hlle", "supersonic-rusanov"])
def test_implicit_step_matches_oracle(ty, golden_dir, case):
    md, om, g, s = setup(ty, golden_dir, case, perturb=0.05)
    nci, nfi = md.ncell_int, md.nface_int
    U0 = g.get_cons()
    st = g.implicit_step(5.0, "GMRES", nkrylov=20, max_it=20, inv_res=1e-10)
    info, it, l1 = s.implicit_step(5.0, nkrylov=20, max_it=20, inv_res=1e-10)
    for name in ("jacL", "jacR"):
        assert close(g.implicit_get(name), s.get_implicit(name)), name
    assert close(g.implicit_get("diag"), s.get_implicit("diag")[:nci])
    assert close(g.implicit_get("upper"), s.get_implicit("upper")[:nfi])
    assert close(g.implicit_get("rhs"), s.implicit_rhs()[:nci])
    du = g.get_cons() - U0
    du_o = s.get("cons")[:, :nci] - U0
    assert np.linalg.norm(du - du_o) <= 1e-9 * np.linalg.norm(du_o)
    assert st["restarts"] == it
    # the boundary face fluxes of that step's right-hand side (F S, as integ_ustboco sums them)
    assert close(g.debug("flux"), s.get("flux"), 1e-12)


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_gmres_golden_history(ty, golden_dir, mode):
    md, om, g, s = setup(ty, golden_dir, GMRES_CASE, mode=mode)
    out = g.ns_steady(10.0, 10.0, cycle_res=0.3, global_res=1e-4, inversion="GMRES", nkrylov=10, max_it=50,
                      inv_res=1e-4, history="RIGHT")
    gold = np.array([[float(x) for x in ln.split()[1:]] for ln in open(golden_dir / "IMPLICIT-GMRES__histofluxNS_RIGHT")
                     if not ln.startswith("#")])
    assert out["flux"].shape == gold.shape == (7, 5)
    for c in range(7):
        assert ["%.5E" % v for v in out["flux"][c]] == ["%.5E" % v for v in gold[c]], c
    g.close()


def test_bicgstab_step_matches_oracle(ty, golden_dir):
    md, om, g, s = setup(ty, golden_dir, SUPERSONIC_CASE, perturb=0.05)
    s.set_inversion("BICGSTAB")
    nci = md.ncell_int
    U0 = g.get_cons()
    st = g.implicit_step(8.0, "BICGSTAB", max_it=50, inv_res=1e-8)
    info, it, l1 = s.implicit_step(8.0, max_it=50, inv_res=1e-8)
    du = g.get_cons() - U0
    du_o = s.get("cons")[:, :nci] - U0
    assert st["info"] >= 0 and info >= 0
    assert abs(st["restarts"] - it) <= 1          # iterations, up to a tie at the stopping test
    assert np.linalg.norm(du - du_o) <= 1e-7 * np.linalg.norm(du_o)
    assert st["lin_res"] < 1e-6


def test_bicgstab_golden_run(ty, golden_dir):
    """NRG/TIME/IMPLICIT/BICGSTAB-RUSANOV on the GPU: fifteen cycles as in the golden file,
    and the converged state of the oracle's run."""
    md, om, g, s = setup(ty, golden_dir, SUPERSONIC_CASE)
    out = g.ns_steady(2.0, 50.0, cycle_res=0.3, global_res=1e-12, inversion="BICGSTAB", max_it=50, inv_res=1e-1)
    s.set_inversion("BICGSTAB")
    lr, _, _, end = s.typhon_steady(2.0, 50.0, cycle_res=0.3, global_res=1e-12, max_it=50, inv_res=1e-1)
    assert len(out["cycle_end"]) == len(end) == 15
    nci = md.ncell_int
    U, Uo = g.get_cons(), s.get("cons")[:, :nci]
    for v in range(5):
        assert np.abs(U[v] - Uo[v]).max() <= 1e-9 * np.abs(Uo[v]).max() + 1e-12, v
    g.close()
