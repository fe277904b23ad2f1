"""The oracle's implicit step (backward Euler, BDLU matrix, restarted GMRES) checked on its own.

Typhon's implicit non-regression cases (NRG/TIME/IMPLICIT) run on CGNS meshes with
inlet/outlet conditions that this path does not carry, so no golden monitor pins the implicit
step.  These tests check the restatement against the mathematics instead:

* the BDLU operator is I - dR/dU: with the Rusanov flux and its Jacobian on a uniform state
  (where the frozen spectral radius is exact) it matches a central finite difference of the
  residual, on periodic and on symmetry boundaries (ns_bocojacobian's mirror);
* GMRES (bdlu_gmres.f90) solves the assembled system: against a dense solve;
* repeated implicit steps at a large CFL drive an isentropic vortex at rest to its discrete
  steady state.
"""
import numpy as np
import pytest

import oracle_py as op

SYMMETRY_BOX = [(f, op.BC_SYMMETRY, "", (0.0, 0.0, 0.0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX")]


def _mesh(golden_dir, name, bcs):
    return op.Mesh.from_tym(golden_dir / name).build(2, bcs)


def _uniform_prim(n, u=0.0, v=0.0):
    return np.stack([np.full(n, 1.2), np.full(n, 1.0 / 1.4), np.full(n, u), np.full(n, v), np.zeros(n)])


def _fd_operator(s, U0, dt, x, eps):
    """x - (R(U0 + eps x) - R(U0 - eps x)) / (2 eps) on interior cells, R at a fixed dtloc."""
    nci = s.mesh.ncell_int
    Rs = []
    for sgn in (1.0, -1.0):
        U = U0.copy()
        U[:, :nci] += sgn * eps * x[:, :nci]
        s.set_cons(U)
        s.rhs(dt)
        Rs.append(s.get("residu")[:, :nci].copy())
    return x[:, :nci] - (Rs[0] - Rs[1]) / (2 * eps)


@pytest.mark.parametrize("name,bcs,u", [("quad10x10.tym", op.PERIODIC_UNIT_SQUARE, 0.3),
                                        ("quad20x10.tym", SYMMETRY_BOX, 0.0)])
def test_bdlu_is_linearised_residual(golden_dir, oracle, name, bcs, u):
    m = _mesh(golden_dir, name, bcs)
    nc, nci = m.ncell, m.ncell_int
    s = op.Solver(m, op.SCH_RUSANOV, op.HRES_NONE, op.LIM_NONE, cfl=1.0)
    s.set_prim(_uniform_prim(nc, u, 0.1 * u))
    U0 = s.get("cons").copy()
    s.implicit_step(3.0)
    dt = s.get("dtloc")[0, 0]
    rng = np.random.default_rng(7)
    x = rng.standard_normal((5, nc))
    x[:, nci:] = 0.0
    fd = _fd_operator(s, U0, dt, x, 1e-6)
    # Typhon's implicit operator keeps each ghost cell as its own unknown (identity row, zero
    # right-hand side): a periodic ghost is not tied to the cell it copies.  The finite
    # difference sees that tie, so give each periodic ghost the value of its source cell.
    ex = m.export()
    xp = x.copy()
    for f in range(m.nface_int, m.nface):
        if ex["face_bckind"][f] == op.BC_PERIODIC:
            xp[:, ex["fc2"][f]] = x[:, ex["fc1"][ex["face_partner"][f]]]
    Ax = s.bdlu_matvec(np.ascontiguousarray(xp.T)).T[:, :nci]
    err = np.linalg.norm(Ax - fd) / np.linalg.norm(fd)
    assert err < 1e-5, err          # O(eps): the spectral radius max() has a kink at a uniform state
    # ghost rows are identity and decoupled
    xg = np.zeros((nc, 5))
    xg[nci:] = 1.0
    y = s.bdlu_matvec(xg)
    assert np.array_equal(y[nci:], xg[nci:])


def _dense(s, nc):
    cols = []
    for j in range(5 * nc):
        e = np.zeros(5 * nc)
        e[j] = 1.0
        cols.append(s.bdlu_matvec(e.reshape(nc, 5)).ravel())
    return np.array(cols).T


@pytest.mark.parametrize("scheme", [op.SCH_HLLC, op.SCH_RUSANOV, op.SCH_ROE])
def test_gmres_solves_bdlu_system(golden_dir, oracle, scheme):
    m = _mesh(golden_dir, "quad10x10.tym", op.PERIODIC_UNIT_SQUARE)
    nc, nci = m.ncell, m.ncell_int
    ex = m.export()
    x, y = ex["ccentre"][:, 0] - 0.5, ex["ccentre"][:, 1] - 0.5
    prim = _uniform_prim(nc, 0.2, 0.1)
    prim[0] += 0.1 * np.exp(-(x * x + y * y) / 0.02)
    runs = []
    for _ in range(2):               # the same step twice is bit for bit the same
        s = op.Solver(m, scheme, op.HRES_NONE, op.LIM_NONE, cfl=1.0)
        s.set_prim(prim)
        U0 = s.get("cons").copy()
        info, it, _ = s.implicit_step(50.0, local_dt=True, nkrylov=30, max_it=50, inv_res=1e-12)
        assert info >= 0 and it >= 1
        runs.append(s.get("cons").copy())
    assert np.array_equal(runs[0], runs[1])
    dU = (runs[1] - U0)[:, :nci]
    dt = s.get("dtloc")[0].copy()
    A = _dense(s, nc)
    R = _residual_local_dt(m, scheme, U0, dt)
    xs = np.linalg.solve(A, np.ascontiguousarray(R.T).ravel()).reshape(nc, 5).T[:, :nci]
    err = np.linalg.norm(dU - xs) / np.linalg.norm(xs)
    assert err < 1e-9, err


def _residual_local_dt(m, scheme, U0, dt):
    """Residual with Typhon's local time steps dt (ncell), ghost rows zero."""
    s = op.Solver(m, scheme, op.HRES_NONE, op.LIM_NONE, cfl=1.0)
    s.set_cons(U0)
    s.rhs(1.0)                        # dtloc = 1: R = -sum F S / V
    R = s.get("residu").copy()
    nci = m.ncell_int
    R[:, :nci] *= dt[:nci]
    R[:, nci:] = 0.0
    return R


def test_implicit_steps_converge_vortex_at_rest(golden_dir, oracle):
    m = _mesh(golden_dir, "quad20x20.tym", op.PERIODIC_UNIT_SQUARE)
    ex = m.export()
    x, y = ex["ccentre"][:, 0] - 0.5, ex["ccentre"][:, 1] - 0.5
    r2 = (x * x + y * y) / 0.01
    n = m.ncell
    prim = np.stack([np.ones(n), 1 / 1.4 - 0.00045 * np.exp(-r2), -0.3 * y * np.exp(-r2 / 2),
                     0.3 * x * np.exp(-r2 / 2), np.zeros(n)])
    s = op.Solver(m, op.SCH_HLLC, op.HRES_NONE, op.LIM_NONE, cfl=1.0)
    s.set_prim(prim)
    hist = []
    for _ in range(12):
        info, _, l1 = s.implicit_step(100.0, local_dt=True, nkrylov=30, max_it=50, inv_res=1e-6)
        assert info >= 0
        hist.append(l1.sum())
    assert hist[-1] < 0.05 * hist[0], hist


FARFIELD_BOX = [(f, op.BC_FARFIELD, "", (0.0, 0.0, 0.0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX")]


def test_farfield_states():
    """The four far-field kinds of the free-stream normal velocity."""
    g = 1.4
    qinf = np.array([1.0, 1.0 / g, 0.5, 0.0, 0.0])      # c = 1, M = 0.5 along x
    q = np.array([2.0, 3.0, 0.1, 0.2, 0.3])
    cases = {(-1.0, 0.0): [1.0, 3.0, 0.5, 0.0, 0.0],     # subsonic inflow: inside pressure
             (1.0, 0.0): [2.0, 1.0 / g, 0.1, 0.2, 0.3],  # subsonic outflow: free-stream pressure
             (0.0, 1.0): [2.0, 1.0 / g, 0.1, 0.2, 0.3],  # vn = 0 counts as outflow
             (0.0, -1.0): [2.0, 1.0 / g, 0.1, 0.2, 0.3]}
    m = op.Mesh.from_tym(__import__("pathlib").Path(__file__).parent / "golden" / "quad10x10.tym").build(
        2, FARFIELD_BOX)
    ex = m.export()
    s = op.Solver(m, op.SCH_RUSANOV, cfl=1.0, farfield=tuple(qinf))
    prim = np.tile(q[:, None], (1, m.ncell))
    s.set_prim(prim)
    s.rhs(1e-3)
    right = s.get("cell_r")                  # face-state mode: the ghost state of each boundary face
    for f in range(m.nface_int, m.nface):
        n = tuple(np.round(ex["fnormal"][f, :2], 12) + 0.0)
        assert n in cases
        assert np.allclose(right[:, f], cases[n], rtol=0, atol=1e-15), (n, right[:, f])
    sup = op.Solver(m, op.SCH_RUSANOV, cfl=1.0, farfield=(1.0, 1.0 / g, 3.0, 0.0, 0.0))   # M = 3
    sup.set_prim(prim)
    sup.rhs(1e-3)
    rs = sup.get("cell_r")
    for f in range(m.nface_int, m.nface):
        nx = ex["fnormal"][f, 0]
        want = [1.0, 1.0 / g, 3.0, 0.0, 0.0] if nx < -0.5 else (q if nx > 0.5 else [2.0, 1.0 / g, 0.1, 0.2, 0.3])
        assert np.allclose(rs[:, f], want, rtol=0, atol=1e-15)


def test_farfield_newton_convergence(golden_dir, oracle):
    """Rusanov with its own Jacobian through far-field boundaries: the implicit step is a
    Newton step as the CFL grows, and a perturbed free stream converges to machine zero."""
    m = _mesh(golden_dir, "quad20x20.tym", FARFIELD_BOX)
    ex = m.export()
    x, y = ex["ccentre"][:, 0] - 0.5, ex["ccentre"][:, 1] - 0.5
    b = 0.1 * np.exp(-(x * x + y * y) / 0.02)
    n = m.ncell
    qinf = (1.0, 1.0 / 1.4, 0.5, 0.1, 0.0)
    prim = np.stack([1 + b, (1 + b) / 1.4, np.full(n, 0.5), 0.1 + b, np.zeros(n)])
    s = op.Solver(m, op.SCH_RUSANOV, cfl=1.0, farfield=qinf)
    s.set_prim(prim)
    cfl, hist = 10.0, []
    for _ in range(16):
        info, _, l1 = s.implicit_step(cfl, local_dt=True, nkrylov=50, max_it=10, inv_res=1e-8)
        hist.append(l1.sum())
        cfl = min(2 * cfl, 1e6)
    assert hist[-1] < 1e-11 * hist[0], hist
    assert np.allclose(s.get("prim")[:, :m.ncell_int], np.array(qinf)[:, None], atol=1e-10)
