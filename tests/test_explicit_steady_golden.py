"""Typhon's steady explicit MUSCL runs on expansion-10.cgns, its VTK output and its volume
probes, without a GPU.

NRG/NS/NUM/HRES/MUSCL: a supersonic expansion (Mach 2 inlet at Pi 1e5, Ti 400; supersonic
outlet; symmetry walls), started from Pi 1e5, Ti 300, Mach 2; TIME = STEADY with the
default METHOD = EXPLICIT (forward Euler) and global stability time step at CFL 1; least-
squares gradients.

* HLLC-MUSCL (HLLC, MUSCL, van Leer), AUSM-MUSCLFAST (AUSM-M, MUSCL-FAST, van Albada),
  NS/NUM/FLUX/HLLC-MUSCLUNS (HLLC, MUSCL-UNS, van Leer, to 1e-3) and NS/HLLC-MPI (HLLC,
  first order; Typhon ran it on two MPI ranks): the oracle's residual history equals
  monres.001 (every iteration, 15 printed digits, to 1e-10 in log10) and ends at the same
  iteration.
* NS/NUM/FLUX/HLLE on square-quad10.cgns (HLLE, subsonic inlets and outlet, RESIDUALS 0.3
  per cycle, 1e-4 overall): after each of the eight cycles the outlet's summed fluxes and
  S-weighted ghost primitive averages equal histofluxNS_RIGHT and histovarNS_RIGHT as
  printed (six digits).
* AUSM-MUSCLFAST's VTK output (typhonNS.vtk): the writer reproduces Typhon's file byte for
  byte from the oracle's state (mesh, cell types, RHO, PS, V).
* AUSM-MUSCLUNS (MUSCL-UNS, run to 1e-6): the VOL_MIN of sqrt(PS), VOL_MAX of V and
  VOL_AVERAGE of V_Y-V_X equal MINP/MAXV/VCOMP.tmon as printed (8 digits).

The VTK file and the probes are of the final state (159 and 461 iterations); its primitive
variables are computed from the conservative state as calc_varprim_ns.f90 does (the
oracle's own primitive array is that of the state the last residual was evaluated on).
"""
import numpy as np
import pytest

import oracle_py as op
from typhon_gb300 import cgns, probes, vtk

GAMMA, RGAS = 1.4, 287.14
Z3 = (0.0, 0.0, 0.0)
INLET = (1e5, 400.0, 2.0, 1.0, 0.0, 0.0)        # PI, TI, MACH, DIRECTION
BCS = [("WALL", op.BC_SYMMETRY, None), ("INLET", op.BC_INLET_SUP, INLET), ("OUTLET", op.BC_OUTLET_SUP, None)]
CASES = {"HLLC-MUSCL": (op.SCH_HLLC, op.HRES_MUSCL, op.LIM_VLEER, 1e-2),
         "HLLC-MUSCLUNS": (op.SCH_HLLC, op.HRES_MUSCLUNS, op.LIM_VLEER, 1e-3),
         "HLLC-MPI": (op.SCH_HLLC, op.HRES_NONE, op.LIM_ALBADA, 1e-2),
         "AUSM-MUSCLFAST": (op.SCH_AUSMM, op.HRES_MUSCLFAST, op.LIM_ALBADA, 1e-2),
         "AUSM-MUSCLUNS": (op.SCH_AUSMM, op.HRES_MUSCLUNS, op.LIM_ALBADA, 1e-6)}


def init_state(pi, ti, mach):
    g = GAMMA
    gmusd, gsgmu = (g - 1.0) / 2.0, g / (g - 1.0)
    p = pi / (1.0 + gmusd * mach ** 2) ** gsgmu
    rho = p / (RGAS * ti) * (1.0 + gmusd * mach ** 2)
    return rho, p, np.sqrt(g * p / rho) * mach


def oracle_case(golden_dir, name):
    raw = cgns.read_cgns(golden_dir / "expansion-10.cgns")
    ob = [(f, k, "", Z3, Z3, d) if d else (f, k, "", Z3) for f, k, d in BCS]
    om = op.Mesh.from_raw(raw).build(2, ob)
    sch, hres, lim, res = CASES[name]
    s = op.Solver(om, sch, highres=hres, limiter=lim, gradmeth=op.GRAD_LSQ if hres else op.GRAD_NONE, gamma=GAMMA,
                  rgas=RGAS, rk="EXPLICIT")
    rho, p, u = init_state(1e5, 300.0, 2.0)
    prim = np.zeros((5, om.ncell))
    prim[0], prim[1], prim[2] = rho, p, u
    s.set_prim(prim)
    lr, _, _, end = s.typhon_steady(1.0, 1.0, cycle_res=res, global_res=res, method="EXPLICIT", max_iters=20000)
    return raw, om, s, lr, end


def prim_of(cons, gamma=GAMMA):
    """calc_varprim_ns.f90:43-54 in the same operation order."""
    rho = cons[0]
    u, v, w = cons[2] / rho, cons[3] / rho, cons[4] / rho
    ec = 0.5 * rho * (u * u + v * v + w * w)
    return np.array([rho, (gamma - 1.0) * (cons[1] - ec), u, v, w])


def test_reads_expansion_mesh(golden_dir):
    raw = cgns.read_cgns(golden_dir / "expansion-10.cgns")
    assert raw.vtex.shape == (118, 3)
    assert sum(len(ie) for t, ie, _ in raw.sections if t != op_bar2()) == 99
    assert [(m[0], len(m[1])) for m in raw.marks] == [("WALL", 13), ("INLET", 16), ("OUTLET", 15)]


def op_bar2():
    from typhon_gb300.umesh import ELEM_BAR2
    return ELEM_BAR2


@pytest.mark.parametrize("name,niter", [("HLLC-MUSCL", 152), ("AUSM-MUSCLFAST", 159), ("HLLC-MUSCLUNS", 227),
                                        ("HLLC-MPI", 174)])
def test_oracle_reproduces_monres(golden_dir, name, niter):
    _, _, _, lr, end = oracle_case(golden_dir, name)
    gold = np.loadtxt(golden_dir / f"{name}__monres.001")
    assert len(lr) == len(gold) == niter and list(end) == [niter]
    assert np.array_equal(gold[:, 0], np.arange(1, niter + 1))
    assert np.abs(lr - gold[:, 1]).max() < 1e-10


def test_vtk_writer_reproduces_typhon_file(golden_dir, tmp_path):
    raw, om, s, _, _ = oracle_case(golden_dir, "AUSM-MUSCLFAST")
    q = prim_of(s.get("cons")[:, :om.ncell_int])
    out = tmp_path / "typhonNS.vtk"
    vtk.write_vtk(out, raw, scalars=[("RHO", q[0]), ("PS", q[1])], vectors=[("V", q[2:5])])
    assert out.read_bytes() == (golden_dir / "AUSM-MUSCLFAST__typhonNS.vtk").read_bytes()
    # the binary form carries the same numbers
    outb = tmp_path / "typhonNS-bin.vtk"
    vtk.write_vtk(outb, raw, scalars=[("RHO", q[0]), ("PS", q[1])], vectors=[("V", q[2:5])], binary=True)
    b = outb.read_bytes()
    head = b"# vtk DataFile Version 2.0\nTYPHON\nBINARY\nDATASET UNSTRUCTURED_GRID\nPOINTS       118 double\n"
    assert b.startswith(head)
    pts = np.frombuffer(b[len(head):len(head) + 118 * 24], ">f8").reshape(118, 3)
    assert np.array_equal(pts, raw.vtex)
    k = b.index(b"SCALARS RHO double\nLOOKUP_TABLE default\n") + len("SCALARS RHO double\nLOOKUP_TABLE default\n")
    order = np.concatenate([ie for t, ie, _ in raw.sections if t != op_bar2()]) - 1
    assert np.array_equal(np.frombuffer(b[k:k + 99 * 8], ">f8"), q[0][order])


def test_fortran_number_format():
    assert vtk.fortran_e(0.1) == "  1.00000000E-001"
    assert vtk.fortran_e(-1.0e-100) == " -1.00000000E-100"
    assert vtk.fortran_e(0.0) == "  0.00000000E+000"
    assert vtk.fortran_e(12345.678) == "  1.23456780E+004"


def test_oracle_reproduces_probes(golden_dir):
    _, om, s, lr, end = oracle_case(golden_dir, "AUSM-MUSCLUNS")
    assert list(end) == [461]
    q = prim_of(s.get("cons")[:, :om.ncell_int])
    ex = om.export()
    env = probes.ns_environment(q, ex["ccentre"][:om.ncell_int])
    vol = ex["cvol"][:om.ncell_int]
    for name, kind, expr in (("MINP", "VOL_MIN", "sqrt(PS)"), ("MAXV", "VOL_MAX", "V"),
                             ("VCOMP", "VOL_AVERAGE", "V_Y-V_X")):
        gold = open(golden_dir / f"AUSM-MUSCLUNS__{name}.tmon").read().split()
        assert gold[:2] == ["1", "0.00000000E+00"]
        v = probes.vol_probe(kind, expr, env, vol)
        assert "%.7E" % v == "%.7E" % float(gold[2]), (name, v, gold[2])


def test_probe_expressions():
    env = probes.ns_environment(np.array([[1.0, 2.0], [4.0, 9.0], [3.0, 0.0], [4.0, 1.0], [0.0, 0.0]]),
                                np.array([[0.0, 1.0, 2.0], [3.0, 4.0, 5.0]]))
    vol = np.array([1.0, 3.0])
    assert probes.vol_probe("VOL_MIN", "sqrt(PS)", env, vol) == 2.0
    assert probes.vol_probe("VOL_MAX", "V", env, vol) == 5.0
    assert probes.vol_probe("vol_average", "V_Y-V_X", env, vol) == 1.0
    assert probes.vol_probe("VOL_AVERAGE", "rho*x + 2", env, vol) == pytest.approx((1 * 0 + 2 + 3 * (2 * 3 + 2)) / 4)
    for bad in ("__import__('os')", "PS.real", "[PS]", "Q + 1"):
        with pytest.raises(probes.ProbeError):
            probes.evaluate(bad, env)


HLLE_BCS = [("LEFT-UP", op.BC_INLET_SUB, (1.7e5, 200.0, 1.0, 0.0, 0.0)),
            ("LEFT-DOWN", op.BC_INLET_SUB, (1.2e5, 600.0, 1.0, 0.0, 0.0)),
            ("RIGHT", op.BC_OUTLET_SUB, (1e5,)), ("TOP", op.BC_SYMMETRY, None), ("BOTTOM", op.BC_SYMMETRY, None)]


def read_histo(path):
    return np.array([[float(x) for x in ln.split()[1:]] for ln in open(path) if not ln.startswith("#")])


def test_oracle_reproduces_hlle_histories(golden_dir):
    import typhon_gb300 as ty
    raw = cgns.read_cgns(golden_dir / "square-quad10.cgns")
    ob = [(f, k, "", Z3, Z3, d) if d else (f, k, "", Z3) for f, k, d in HLLE_BCS]
    om = op.Mesh.from_raw(raw).build(2, ob)
    md = ty.preprocess(raw, 2, [(f, k, "", Z3) for f, k, _ in HLLE_BCS])
    s = op.Solver(om, op.SCH_HLLE, gamma=GAMMA, rgas=RGAS, rk="EXPLICIT")
    rho, p, u = init_state(1e5, 300.0, 2.0)
    prim = np.zeros((5, om.ncell))
    prim[0], prim[1], prim[2] = rho, p, u
    s.set_prim(prim)
    lr, fs, ga, end = s.typhon_steady(1.0, 1.0, cycle_res=0.3, global_res=1e-4, method="EXPLICIT",
                                      history_faces=md.faces_of("RIGHT"))
    gf = read_histo(golden_dir / "HLLE-EXPLICIT__histofluxNS_RIGHT")
    gv = read_histo(golden_dir / "HLLE-EXPLICIT__histovarNS_RIGHT")
    assert len(end) == len(gf) == len(gv) == 8
    for c in range(8):
        assert ["%.5E" % v for v in fs[c]] == ["%.5E" % v for v in gf[c]], c
        assert ["%.5E" % v for v in ga[c]] == ["%.5E" % v for v in gv[c]], c


def test_oracle_local_time_step_converges_faster(golden_dir):
    """DTCALC = LOCAL_STABILITY_CONDITION on HLLC-MUSCL's case: per-cell time steps reach the
    same 1e-2 residual drop in fewer iterations than the global one (152)."""
    raw = cgns.read_cgns(golden_dir / "expansion-10.cgns")
    ob = [(f, k, "", Z3, Z3, d) if d else (f, k, "", Z3) for f, k, d in BCS]
    om = op.Mesh.from_raw(raw).build(2, ob)
    s = op.Solver(om, op.SCH_HLLC, highres=op.HRES_MUSCL, limiter=op.LIM_VLEER, gradmeth=op.GRAD_LSQ, gamma=GAMMA,
                  rgas=RGAS, rk="EXPLICIT")
    rho, p, u = init_state(1e5, 300.0, 2.0)
    prim = np.zeros((5, om.ncell))
    prim[0], prim[1], prim[2] = rho, p, u
    s.set_prim(prim)
    lr, _, _, end = s.typhon_steady(1.0, 1.0, cycle_res=1e-2, global_res=1e-2, method="EXPLICIT", local_dt=True)
    assert 0 < end[0] < 152
    assert lr[-1] - lr.max() <= -2.0
