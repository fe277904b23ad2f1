"""The heat-conduction (KDIF) oracle checked on its own.

Typhon's KDIF non-regression cases run on CGNS meshes, so the restatement of
calc_kdif_flux / kdif_bocoflux / the implicit step is checked against the mathematics: a
linear temperature field is conducted exactly by the full and cell-average face gradients
(zero balance in cells away from boundaries); conjugate gradients agree with a dense solve
of the assembled system; implicit steps reach the steady profile between two isothermal
walls, symmetric about the middle plane.
"""
import numpy as np
import pytest

import oracle_py as op
from typhon_gb300 import umesh

BOX = [("IMIN", umesh.BC_WALL, "", (0, 0, 0)), ("IMAX", umesh.BC_WALL, "", (0, 0, 0)),
       ("JMIN", umesh.BC_WALL, "", (0, 0, 0)), ("JMAX", umesh.BC_WALL, "", (0, 0, 0)),
       ("KMIN", umesh.BC_WALL, "", (0, 0, 0)), ("KMAX", umesh.BC_WALL, "", (0, 0, 0))]


def box(n, jitter):
    raw = umesh.gen_tet_box(n, 1.0, jitter=jitter, seed=5)
    m = op.Mesh.from_raw(raw).build(3, BOX)
    ex = m.export()
    kind = np.zeros(m.nface, np.int32)
    value = np.zeros(m.nface)
    fc = ex["fcentre"]
    for f in range(m.nface_int, m.nface):
        if abs(fc[f, 0]) < 1e-12:
            kind[f], value[f] = op.KBC_ISOTHERMAL, 0.0
        elif abs(fc[f, 0] - 1.0) < 1e-12:
            kind[f], value[f] = op.KBC_ISOTHERMAL, 1.0
        else:
            kind[f], value[f] = op.KBC_FLUX, 0.0
    return m, ex, kind, value


@pytest.mark.parametrize("scheme", [op.KDIF_FULL, op.KDIF_CELLAVG])
def test_linear_field_is_conducted_exactly(oracle, scheme):
    m, ex, kind, value = box(6, 0.1)
    k = op.Kdif(m, scheme, 2.0, np.full(m.ncell_int, 3.0), kind, value)
    T = 0.3 + 2.0 * ex["ccentre"][:, 0] - 0.5 * ex["ccentre"][:, 1] + 0.7 * ex["ccentre"][:, 2]
    k.set_T(T)
    k.rhs(1.0)
    g = k.get("grad")[:, :m.ncell_int]
    inner = np.ones(m.ncell_int, bool)               # cells with no boundary face
    for f in range(m.nface_int, m.nface):
        inner[ex["fc1"][f]] = False
    assert np.allclose(g[:, inner].T, [2.0, -0.5, 0.7], atol=1e-12)
    inner2 = inner.copy()                            # ... and no neighbour with one
    for f in range(m.nface_int):
        a, b = ex["fc1"][f], ex["fc2"][f]
        if not (inner[a] and inner[b]):
            inner2[a] = inner2[b] = False
    assert inner2.sum() > 0
    inner = inner2
    bal = k.get("balance")
    flux_scale = 3.0 * 2.2 * np.abs(ex["fsurf"]).max()
    assert np.abs(bal[inner]).max() < 1e-12 * flux_scale


def test_cg_matches_dense_solve(oracle):
    m, ex, kind, value = box(4, 0.1)
    rng = np.random.default_rng(2)
    kc = np.exp(rng.standard_normal(m.ncell_int))
    k = op.Kdif(m, op.KDIF_FULL, 1.5, kc, kind, value)
    k.set_T(rng.uniform(0, 1, m.ncell))
    k.rhs(1e-2)
    k.assemble(1e-2)
    n = m.ncell_int
    A = np.array([k.matvec(np.eye(n)[j]) for j in range(n)]).T
    assert np.allclose(A, A.T, rtol=1e-13, atol=0)
    assert np.all(np.linalg.eigvalsh(A) > 0)
    b = k.get("balance")
    T0 = k.get("T")[:n].copy()
    it, rel = k.implicit_step(1e-2, tol=1e-13)
    assert rel < 1e-13
    dT = (k.get("T")[:n] - T0) * 1.5
    assert np.allclose(dT, np.linalg.solve(A, b), rtol=1e-9, atol=1e-12)


def test_steady_profile_between_isothermal_walls(oracle):
    m, ex, kind, value = box(6, 0.0)
    k = op.Kdif(m, op.KDIF_FULL, 1.0, np.ones(m.ncell_int), kind, value)
    k.set_T(np.full(m.ncell, 0.5))
    for _ in range(6):
        k.implicit_step(1e6, tol=1e-13)
    k.rhs(1.0)
    n = m.ncell_int
    x = ex["ccentre"][:n, 0]
    T = k.get("T")[:n]
    assert np.abs(k.get("balance")).max() < 1e-8
    # close to linear in x (the wall temperature sits on the mirrored ghost centre, one cell
    # beyond the wall), and T(x) + T(1 - x) = 1 on average by the mesh's symmetry
    a, b0 = np.polyfit(x, T, 1)
    assert a > 0.7 and np.abs(T - (a * x + b0)).max() < 0.01
    assert abs(T.mean() - 0.5) < 1e-9
