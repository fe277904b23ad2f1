"""The implicit oracle against Typhon's own implicit golden runs, without a GPU.

NRG/TIME/IMPLICIT/GMRES: square-quad10.cgns (100 quads), Euler, HLLE flux with the HLL
Jacobian, two subsonic inlets, a subsonic outlet (SAVE_HISTORY = QUANTITY-FLUX) and two
symmetry planes, steady, CFL 10, backward Euler with Typhon's GMRES (NKRYLOV 10, INV_RES
1e-4), 0.3 residual drop per cycle to 1e-4 overall, initial state PI 1e5, TI 300, Mach 2.
The oracle's restatement (mesh, ghost faces, HLLE, boundary states, flux Jacobians, BDLU
assembly, GMRES, the steady driver's CFL law and residual, integ_ustboco's sums) reproduces
every printed digit of both history files over the seven cycles.

NRG/TIME/IMPLICIT/BICGSTAB-RUSANOV (rect4x1.cgns, Rusanov, supersonic inlets and outlet,
Typhon's BiCGSTAB with the CFL ramp from 2 to 50) writes only the S-weighted average of the
ghost state at a symmetry plane, which first-order runs never update: the file pins the
Mach-4 initial state (init_ns_ust.f90) and, by its length, the fifteen cycles the run takes.
"""
import numpy as np

import oracle_py as op
from typhon_gb300 import cgns

GAMMA, RGAS = 1.4, 287.14   # GAS = AIR (def_model_ns.f90:148-154)


def init_state(pi, ti, mach, direction=(1.0, 0.0, 0.0)):
    """INIT block with PI, TI, MACH, DIRECTION (init_ns_ust.f90:118-140)."""
    g = GAMMA
    gmusd, gsgmu = (g - 1.0) / 2.0, g / (g - 1.0)
    p = pi / (1.0 + gmusd * mach ** 2) ** gsgmu
    rho = p / (RGAS * ti) * (1.0 + gmusd * mach ** 2)
    vel = np.sqrt(g * p / rho) * mach
    d = np.asarray(direction, float)
    u = (vel / np.sqrt(np.sum(d * d))) * d
    return rho, p, u


def read_history(path):
    return np.array([[float(x) for x in ln.split()[1:]] for ln in open(path) if not ln.startswith("#")])


def fortran_e(x):
    """Typhon's 1e14.6 field: 0.dddddd E+xx, six significant digits."""
    return "%.5E" % x


def test_gmres_case_boundary_histories(golden_dir):
    raw = cgns.read_cgns(golden_dir / "square-quad10.cgns")
    z3 = (0.0, 0.0, 0.0)
    bcs = [("LEFT-UP", op.BC_INLET_SUB, "", z3, z3, (1.7e5, 200.0, 1.0, 0.0, 0.0)),
           ("LEFT-DOWN", op.BC_INLET_SUB, "", z3, z3, (1.2e5, 600.0, 1.0, 0.0, 0.0)),
           ("RIGHT", op.BC_OUTLET_SUB, "", z3, z3, (1e5,)),
           ("TOP", op.BC_SYMMETRY, "", z3), ("BOTTOM", op.BC_SYMMETRY, "", z3)]
    m = op.Mesh.from_raw(raw).build(2, bcs)
    ex = m.export()
    right = [f for f in range(m.nface_int, m.nface) if ex["face_bckind"][f] == op.BC_OUTLET_SUB]
    assert len(right) == 10
    rho, p, u = init_state(1e5, 300.0, 2.0)
    prim = np.zeros((5, m.ncell))
    prim[0], prim[1], prim[2] = rho, p, u[0]
    s = op.Solver(m, op.SCH_HLLE, gamma=GAMMA, rgas=RGAS)
    s.set_prim(prim)
    lr, flux, ghost, end = s.typhon_steady(10.0, 10.0, cycle_res=0.3, global_res=1e-4, nkrylov=10, max_it=50,
                                          inv_res=1e-4, history_faces=right)
    hf = read_history(golden_dir / "IMPLICIT-GMRES__histofluxNS_RIGHT")
    hv = read_history(golden_dir / "IMPLICIT-GMRES__histovarNS_RIGHT")
    assert len(end) == len(hf) == len(hv) == 7
    for c in range(7):
        assert [fortran_e(v) for v in flux[c]] == [fortran_e(v) for v in hf[c]], c
        assert [fortran_e(v) for v in ghost[c]] == [fortran_e(v) for v in hv[c]], c
    assert np.all(np.diff(lr) < 0.5)   # a converging history (no blow-up between cycles)


def test_bicgstab_case_initial_state(golden_dir):
    raw = cgns.read_cgns(golden_dir / "rect4x1.cgns")
    z3 = (0.0, 0.0, 0.0)
    bcs = [("DOWN", op.BC_SYMMETRY, "", z3), ("RIGHT", op.BC_OUTLET_SUP, "", z3),
           ("LEFT", op.BC_INLET_SUP, "", z3, z3, (1e5, 300.0, 4.0, 1.0, 0.0, 0.0)),
           ("UP", op.BC_INLET_SUP, "", z3, z3, (98497.053, 300.0, 3.60110, 1.0, -0.0967742, 0.0))]
    m = op.Mesh.from_raw(raw).build(2, bcs)
    ex = m.export()
    down = [f for f in range(m.nface_int, m.nface) if ex["face_bckind"][f] == op.BC_SYMMETRY]
    rho, p, u = init_state(1e5, 300.0, 4.0)
    hv = read_history(golden_dir / "IMPLICIT-BICGSTAB-RUSANOV__histovarNS_DOWN")
    assert [fortran_e(v) for v in (rho, p, u[0], u[1], u[2])] == [fortran_e(v) for v in hv[0]]
    # the full run: Typhon's BiCGSTAB (its default, INV_RES 1e-1, IMP_MAX_IT 50), CFL 2 ramped
    # to 50 by the residual, RESIDUALS 0.3 per cycle down to 1e-12: fifteen cycles, as the
    # golden file has, each printing the initial ghost state
    prim = np.zeros((5, m.ncell))
    prim[0], prim[1], prim[2] = rho, p, u[0]
    s = op.Solver(m, op.SCH_RUSANOV, gamma=GAMMA, rgas=RGAS)
    s.set_prim(prim)
    s.set_inversion("BICGSTAB")
    lr, flux, ghost, end = s.typhon_steady(2.0, 50.0, cycle_res=0.3, global_res=1e-12, max_it=50, inv_res=1e-1,
                                          history_faces=down)
    assert len(end) == len(hv) == 15
    assert lr[-1] - lr[0] < -12.0
    for c in range(len(end)):
        assert [fortran_e(v) for v in ghost[c]] == [fortran_e(v) for v in hv[c]]
