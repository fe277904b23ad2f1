"""Property pins of the Roe flux on the CPU oracle (Typhon has no Roe flux to compare with:
SOURCE/EQNS/calc_flux_inviscid.f90:48-79 stops on SCHEME = ROE).

The same properties are checked on the GPU kernels in tests/test_gpu_roe_properties.py, and
the GPU agrees with the oracle bit for bit in exact mode (tests/test_gpu_explicit.py), so
these pins hold for both.
"""
import numpy as np
import pytest

import flux_props as fp
import oracle_py as op

N = 4000


@pytest.fixture(scope="module")
def rng():
    return np.random.default_rng(20261204)


def rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1.0)


def test_consistency(rng):
    """F(U, U, n) = F_phys(U).n for subsonic, sonic and supersonic normal velocities."""
    q = fp.random_states(rng, N, speed=3.0)
    n = fp.random_normals(rng, N)
    F = op.roe_flux(q, q, n)
    assert rel(F, fp.physical_flux(q, n)).max() < 1e-14


def test_rotational_invariance(rng):
    """Rotating both states and the normal rotates the momentum flux; mass and energy
    fluxes are unchanged (1e-13: only rounding differs)."""
    qL, qR = fp.random_states(rng, N), fp.random_states(rng, N)
    n = fp.random_normals(rng, N)
    F = op.roe_flux(qL, qR, n)
    for _ in range(3):
        Q = fp.random_rotation(rng)
        Fr = op.roe_flux(fp.rotate_prim(qL, Q), fp.rotate_prim(qR, Q), n @ Q.T)
        scale = np.abs(F).max(axis=1, keepdims=True)
        assert (np.abs(Fr - fp.rotate_flux(F, Q)) / scale).max() < 1e-13


def test_swapping_sides_reverses_the_flux(rng):
    """F(L, R, n) = -F(R, L, -n): the flux through a face does not depend on which cell is
    called left (the basis of discrete conservation)."""
    qL, qR = fp.random_states(rng, N), fp.random_states(rng, N)
    n = fp.random_normals(rng, N)
    F1 = op.roe_flux(qL, qR, n)
    F2 = op.roe_flux(qR, qL, -n)
    scale = np.abs(F1).max(axis=1, keepdims=True)
    assert (np.abs(F1 + F2) / scale).max() < 1e-13


def test_stationary_contact_is_exact(rng):
    """Equal pressure, zero velocity, any density jump: no mass or energy flux, momentum
    flux p n (the entropy fix acts on the acoustic waves only, so the contact is not smeared)."""
    m = 500
    p = rng.uniform(0.5, 2.0, m)
    qL = np.column_stack([rng.uniform(0.2, 5.0, m), p, np.zeros((m, 3))])
    qR = np.column_stack([rng.uniform(0.2, 5.0, m), p, np.zeros((m, 3))])
    n = fp.random_normals(rng, m)
    F = op.roe_flux(qL, qR, n)
    assert np.abs(F[:, 0:2]).max() < 1e-15
    assert np.abs(F[:, 2:5] - p[:, None] * n).max() < 1e-15


def test_moving_contact_is_upwinded_exactly(rng):
    """Equal pressure and velocity, a density jump: the flux is the physical flux of the
    upwind side (Roe's linearisation is exact for an isolated contact)."""
    m = 500
    p = rng.uniform(0.5, 2.0, m)
    u = rng.uniform(-0.8, 0.8, (m, 3))
    qL = np.column_stack([rng.uniform(0.2, 5.0, m), p, u])
    qR = np.column_stack([rng.uniform(0.2, 5.0, m), p, u])
    n = fp.random_normals(rng, m)
    F = op.roe_flux(qL, qR, n)
    vn = np.einsum("ij,ij->i", u, n)
    up = np.where((vn > 0)[:, None], fp.physical_flux(qL, n), fp.physical_flux(qR, n))
    assert rel(F, up).max() < 1e-13


def test_discrete_conservation_periodic_tgv():
    """On the periodic TGV mesh the face fluxes cancel: sum over cells of R V / dt is zero to
    rounding for the benchmark scheme (Roe + MUSCL-UNS + Barth)."""
    import typhon_gb300 as ty
    from typhon_gb300 import cases
    L = 2 * np.pi
    raw = ty.gen_tet_box(6, L, jitter=0.05, seed=1234)
    om = op.Mesh.from_raw(raw).build(3, ty.periodic_box_bcs((L, L, L)))
    d = om.export()
    s = op.Solver(om, op.SCH_ROE, op.HRES_MUSCLUNS, op.LIM_NONE, op.POSTLIM_BARTH, op.GRAD_LSQ, rk="RK3-SSP")
    s.set_prim(cases.taylor_green(d["ccentre"]))
    dt = s.timestep()
    s.rhs(dt)
    nci = om.ncell_int
    RV = s.get("residu")[:, :nci] * d["cvol"][:nci] / dt
    total = np.abs(RV).sum(axis=1)
    assert np.all(np.abs(RV.sum(axis=1)) <= 1e-13 * total), RV.sum(axis=1) / total


def test_isentropic_vortex_second_order():
    """The vortex2d case with the Roe flux (MUSCL, van Albada, RK4) advected for t = 2: the L1
    density error against the translated exact vortex falls at second order (n = 16, 32, 64
    triangles per side; measured orders 1.92 and 2.16)."""
    import typhon_gb300 as ty
    from typhon_gb300 import cases
    T = 2.0
    errs = []
    for n in (16, 32, 64):
        raw = ty.gen_grid2d(n, n, 10.0, 10.0, "tri", jitter=0.1, seed=1234)
        om = op.Mesh.from_raw(raw).build(2, ty.periodic_box_bcs((10.0, 10.0)))
        d = om.export()
        s = op.Solver(om, op.SCH_ROE, op.HRES_MUSCL, op.LIM_ALBADA, op.POSTLIM_NONE, op.GRAD_LSQ, rk="RK4", cfl=0.8)
        s.set_prim(cases.isentropic_vortex(d["ccentre"]))
        ns = int(np.ceil(T / s.timestep()))
        for _ in range(ns):
            s.rk_step(T / ns)
        nci = om.ncell_int
        ex = fp.vortex_exact(cases, d["ccentre"][:nci], T)
        errs.append(fp.l1_density_error(s.get("prim")[0, :nci], ex[0], d["cvol"][:nci]))
    orders = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(orders > 1.8), (errs, orders)
