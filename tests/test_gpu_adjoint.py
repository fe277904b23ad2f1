"""GPU adjoint of the first-order residual and of explicit runs.

* ty_adjoint_vjp against central finite differences of ty_residual_device (periodic,
  symmetry, far-field, slip and no-slip wall boundaries; HLLC, Rusanov, Roe; exact and fast
  modes); the second-order VJP (least-squares gradients, MUSCL, van Albada) likewise on
  periodic meshes, and through a whole unsteady run against the complex step; with Typhon's
  Barth post-limiter frozen (MUSCL-UNS and MUSCL), against the complex step of the numpy
  restatement with the same frozen ratios (finite differences would see the limiter move).
* The gradient of J = sum over a sub-box of rho^2 V after an RK3-SSP run, through
  typhon_gb300.adjoint (binomial checkpointing or stored stage states, torch.autograd),
  against the complex-step derivative of the numpy restatement in tests/residual_cs.py:
  agreement to 1e-8.
"""
import numpy as np
import pytest

import oracle_py as op
import residual_cs as cs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from typhon_gb300 import build
    build.build()
    import typhon_gb300 as ty
    from typhon_gb300 import adjoint
    return torch, ty, adjoint


def jittered(ty, n=10):
    raw = ty.gen_grid2d(n, n, 1.0, 1.0, "tri", jitter=0.1, seed=3)
    return ty.preprocess(raw, 2, op.PERIODIC_UNIT_SQUARE)


def smooth_cons(ty, md, amp=0.1):
    x, y = md.cell_centre[:md.ncell_int, 0], md.cell_centre[:md.ncell_int, 1]
    t = 2 * np.pi
    prim = np.stack([1 + amp * np.sin(t * x + 0.3) * np.sin(t * y + 1.1), (1 + amp * np.cos(t * (x + y))) / 1.4,
                     0.3 + amp * np.sin(t * y + 0.5), 0.2 * np.cos(t * x + 0.7), 0.05 * np.sin(t * x)])
    return ty.prim_to_cons(prim)


CASES = [("periodic", "HLLC"), ("periodic", "RUSANOV"), ("periodic", "ROE"), ("symmetry", "ROE"),
         ("symmetry", "HLLC"), ("farfield", "HLLC"), ("farfield", "ROE"), ("wall", "RUSANOV"),
         ("noslip", "ROE")]
BC_KIND = {"symmetry": op.BC_SYMMETRY, "farfield": op.BC_FARFIELD, "wall": op.BC_WALL, "noslip": op.BC_NOSLIP}


@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("bc,scheme", CASES)
def test_vjp_matches_finite_differences(env, golden_dir, bc, scheme, mode):
    torch, ty, adjoint = env
    if bc == "periodic":
        md = jittered(ty)
    else:
        kind = BC_KIND[bc]
        md = ty.preprocess(ty.read_tym(golden_dir / "quad20x10.tym"), 2,
                           [(f, kind, "", (0.0, 0.0, 0.0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX")])
    g = ty.Grid(md)
    g.set_spat(scheme, mode=mode, farfield=(1.0, 1.0 / 1.4, 0.3, 0.1, 0.0))
    st = adjoint.Stepper(g, "RK3-SSP")
    U = torch.tensor(smooth_cons(ty, md), device="cuda")
    rng = np.random.default_rng(0)
    lamR = torch.tensor(rng.standard_normal(U.shape), device="cuda")
    d = torch.tensor(rng.standard_normal(U.shape), device="cuda") * U.abs().mean(dim=1, keepdim=True)
    dt = 1e-3
    lamU = st.vjp(U, dt, lamR)
    eps = 1e-6
    fd = ((st.residual(U + eps * d, dt) - st.residual(U - eps * d, dt)) * lamR).sum() / (2 * eps)
    ad = (lamU * d).sum()
    assert abs(float(fd - ad)) <= 1e-7 * abs(float(ad)), (float(fd), float(ad))
    g.close()


@pytest.mark.parametrize("scheme", ["RUSANOV", "HLLC", "ROE"])
def test_unsteady_gradient_against_complex_step(env, scheme):
    torch, ty, adjoint = env
    md = jittered(ty, 8)
    g = ty.Grid(md)
    g.set_spat(scheme, mode="exact")
    U0 = smooth_cons(ty, md)
    dts = [2e-3] * 12
    nci = md.ncell_int
    cc = md.cell_centre[:nci]
    box = ((np.abs(cc[:, 0] - 0.5) < 0.25) & (np.abs(cc[:, 1] - 0.5) < 0.25)).astype(float)
    V = md.cell_volume[:nci]
    Ut = torch.tensor(U0, device="cuda", requires_grad=True)
    Uf = adjoint.rk_solve(Ut, g, "RK3-SSP", dts, snaps=3)
    w = torch.tensor(box * V, device="cuda")
    J = (Uf[0] ** 2 * w).sum()
    J.backward()
    grad = Ut.grad.cpu().numpy()
    # the same run on the host, real: the final states agree
    Uf_np = cs.rk_run(md, U0, dts, adjoint.RK_TABLES["RK3-SSP"], scheme)
    assert np.allclose(Uf.detach().cpu().numpy(), Uf_np, rtol=1e-11, atol=0)
    # complex-step directional derivatives
    rng = np.random.default_rng(4)
    for _ in range(3):
        d = rng.standard_normal(U0.shape) * np.abs(U0).mean(axis=1, keepdims=True)
        h = 1e-30
        Uc = cs.rk_run(md, U0 + 1j * h * d, dts, adjoint.RK_TABLES["RK3-SSP"], scheme)
        dJ = float(np.sum(box * V * Uc[0] ** 2).imag / h)
        ad = float(np.sum(grad * d))
        assert abs(ad - dJ) <= 1e-8 * abs(dJ), (ad, dJ)
    # fewer snapshots, same gradient
    Ut2 = torch.tensor(U0, device="cuda", requires_grad=True)
    J2 = (adjoint.rk_solve(Ut2, g, "RK3-SSP", dts, snaps=0)[0] ** 2 * w).sum()
    J2.backward()
    assert torch.allclose(Ut2.grad, Ut.grad, rtol=1e-13, atol=0)
    # every stage state kept by the forward pass: the same gradient, nothing recomputed
    Ut3 = torch.tensor(U0, device="cuda", requires_grad=True)
    J3 = (adjoint.rk_solve(Ut3, g, "RK3-SSP", dts, snaps="stages")[0] ** 2 * w).sum()
    J3.backward()
    assert torch.allclose(Ut3.grad, Ut.grad, rtol=1e-13, atol=0)
    # the default storage policy (a small run: every stage state fits)
    Ut4 = torch.tensor(U0, device="cuda", requires_grad=True)
    J4 = (adjoint.rk_solve(Ut4, g, "RK3-SSP", dts)[0] ** 2 * w).sum()
    J4.backward()
    assert torch.equal(Ut4.grad, Ut3.grad)
    g.close()


def test_adjoint_rejects_unsupported_second_order(env, golden_dir):
    torch, ty, adjoint = env
    md = jittered(ty, 4)
    for highres, limiter, postlim in (("MUSCL-FAST", "ALBADA", "NONE"), ("MUSCL", "MINMOD", "NONE"),
                                      ("MUSCL-UNS", "SUPERBEE", "BARTH"), ("NONE", "NONE", "BARTH")):
        g = ty.Grid(md)
        g.set_spat("HLLC", highres, limiter, postlim)
        st = adjoint.Stepper(g, "RK2")
        U = torch.tensor(smooth_cons(ty, md), device="cuda")
        with pytest.raises(ty.TyphonError):
            st.vjp(U, 1e-3, torch.ones_like(U))
        g.close()
    # MUSCL on a mesh with a non-periodic boundary
    md2 = ty.preprocess(ty.read_tym(golden_dir / "quad20x10.tym"), 2,
                        [(f, op.BC_SYMMETRY, "", (0.0, 0.0, 0.0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX")])
    g = ty.Grid(md2)
    g.set_spat("HLLC", "MUSCL", "ALBADA")
    st = adjoint.Stepper(g, "RK2")
    U = torch.tensor(smooth_cons(ty, md2), device="cuda")
    with pytest.raises(ty.TyphonError):
        st.vjp(U, 1e-3, torch.ones_like(U))
    g.close()


@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("scheme,limiter", [("HLLC", "ALBADA"), ("ROE", "ALBADA"), ("RUSANOV", "NONE")])
def test_muscl_vjp_matches_finite_differences(env, scheme, limiter, mode):
    """Second order (least-squares gradients, MUSCL, van Albada) on a jittered periodic mesh."""
    torch, ty, adjoint = env
    md = jittered(ty)
    g = ty.Grid(md)
    g.set_spat(scheme, "MUSCL", limiter, mode=mode)
    st = adjoint.Stepper(g, "RK3-SSP")
    U = torch.tensor(smooth_cons(ty, md), device="cuda")
    rng = np.random.default_rng(1)
    lamR = torch.tensor(rng.standard_normal(U.shape), device="cuda")
    d = torch.tensor(rng.standard_normal(U.shape), device="cuda") * U.abs().mean(dim=1, keepdim=True)
    dt = 1e-3
    lamU = st.vjp(U, dt, lamR)
    eps = 1e-6
    fd = ((st.residual(U + eps * d, dt) - st.residual(U - eps * d, dt)) * lamR).sum() / (2 * eps)
    ad = (lamU * d).sum()
    assert abs(float(fd - ad)) <= 1e-6 * abs(float(ad)), (float(fd), float(ad))
    g.close()


@pytest.mark.parametrize("scheme", ["HLLC", "ROE"])
def test_muscl_unsteady_gradient_against_complex_step(env, scheme):
    """J = sum over a sub-box of rho^2 V after an SSP-RK3 run with MUSCL + van Albada: the
    adjoint's directional derivatives against the complex step of the numpy restatement."""
    torch, ty, adjoint = env
    md = jittered(ty, 8)
    g = ty.Grid(md)
    g.set_spat(scheme, "MUSCL", "ALBADA", mode="exact")
    U0 = smooth_cons(ty, md)
    dts = [2e-3] * 10
    nci = md.ncell_int
    cc = md.cell_centre[:nci]
    box = ((np.abs(cc[:, 0] - 0.5) < 0.25) & (np.abs(cc[:, 1] - 0.5) < 0.25)).astype(float)
    V = md.cell_volume[:nci]
    Ut = torch.tensor(U0, device="cuda", requires_grad=True)
    Uf = adjoint.rk_solve(Ut, g, "RK3-SSP", dts)
    w = torch.tensor(box * V, device="cuda")
    J = (Uf[0] ** 2 * w).sum()
    J.backward()
    grad = Ut.grad.cpu().numpy()
    Uf_np = cs.rk_run(md, U0, dts, adjoint.RK_TABLES["RK3-SSP"], scheme, highres="MUSCL", limiter="ALBADA")
    assert np.allclose(Uf.detach().cpu().numpy(), Uf_np, rtol=1e-11, atol=0)
    rng = np.random.default_rng(5)
    for _ in range(3):
        d = rng.standard_normal(U0.shape) * np.abs(U0).mean(axis=1, keepdims=True)
        h = 1e-30
        Uc = cs.rk_run(md, U0 + 1j * h * d, dts, adjoint.RK_TABLES["RK3-SSP"], scheme, highres="MUSCL",
                       limiter="ALBADA")
        dJ = float(np.sum(box * V * Uc[0] ** 2).imag / h)
        ad = float(np.sum(grad * d))
        assert abs(ad - dJ) <= 1e-8 * abs(dJ), (ad, dJ)
    g.close()


def test_muscl_tgv3d_gradient_against_complex_step(env):
    """The benchmark's configuration at a small size: Taylor-Green vortex on 6^3 x 5 jittered
    periodic tetrahedra, HLLC with MUSCL and van Albada, 20 SSP-RK3 steps, J = sum over the
    centred sub-box of rho^2 V: adjoint directional derivatives against the complex step."""
    torch, ty, adjoint = env
    from typhon_gb300 import cases
    md = cases.make_mesh("tgv3d", 6)
    nci = md.ncell_int
    g = ty.Grid(md)
    g.set_spat("HLLC", "MUSCL", "ALBADA", mode="fast")
    prim = cases.taylor_green(md.cell_centre)
    U0 = ty.prim_to_cons(prim[:, :nci])
    g.set_prim(prim)
    dt = g.calc_zonetimestep(0.8)
    dts = [dt] * 20
    cc = md.cell_centre[:nci]
    L = 2 * np.pi
    box = np.all(np.abs(cc - L / 2) < L / 4, axis=1).astype(float) * md.cell_volume[:nci]
    Ut = torch.tensor(U0, device="cuda", requires_grad=True)
    J = (adjoint.rk_solve(Ut, g, "RK3-SSP", dts)[0] ** 2 * torch.tensor(box, device="cuda")).sum()
    J.backward()
    grad = Ut.grad.cpu().numpy()
    rng = np.random.default_rng(7)
    for _ in range(2):
        d = rng.standard_normal(U0.shape) * np.abs(U0).mean(axis=1, keepdims=True)
        Uc = cs.rk_run(md, U0 + 1j * 1e-30 * d, dts, adjoint.RK_TABLES["RK3-SSP"], "HLLC", highres="MUSCL",
                       limiter="ALBADA")
        dJ = float(np.sum(box * Uc[0] ** 2).imag / 1e-30)
        ad = float(np.sum(grad * d))
        assert abs(ad - dJ) <= 1e-8 * abs(dJ), (ad, dJ)
    g.close()


@pytest.mark.parametrize("mode", ["exact", "fast"])
@pytest.mark.parametrize("scheme,highres,limiter,postlim", [("ROE", "MUSCL-UNS", "NONE", "BARTH"),
                                                            ("HLLC", "MUSCL-UNS", "ALBADA", "NONE"),
                                                            ("HLLC", "MUSCL", "ALBADA", "SUPERBARTH")])
def test_frozen_barth_vjp_against_complex_step(env, scheme, highres, limiter, postlim, mode):
    """One residual's VJP with the Barth post-limiter frozen at the state's ratios (and
    MUSCL-UNS): lambda_R . (dR/dU d) against the complex step of the numpy restatement, whose
    ratios come from the real parts.  The state is rough enough for the limiter to act."""
    torch, ty, adjoint = env
    md = jittered(ty)
    g = ty.Grid(md)
    g.set_spat(scheme, highres, limiter, postlim, mode=mode)
    st = adjoint.Stepper(g, "RK3-SSP")
    rng = np.random.default_rng(2)
    U0 = smooth_cons(ty, md) * (1.0 + 0.05 * rng.standard_normal((1, md.ncell_int)))
    U = torch.tensor(U0, device="cuda")
    lamR = rng.standard_normal(U0.shape)
    d = rng.standard_normal(U0.shape) * np.abs(U0).mean(axis=1, keepdims=True)
    dt = 1e-3
    lamU = st.vjp(U, dt, torch.tensor(lamR, device="cuda")).cpu().numpy()
    Rc = cs.residual(md, U0 + 1j * 1e-30 * d, dt, scheme, highres=highres, limiter=limiter, postlim=postlim)
    cs_dir = float(np.sum(lamR * Rc.imag) / 1e-30)
    ad = float(np.sum(lamU * d))
    assert abs(ad - cs_dir) <= 1e-9 * abs(cs_dir), (ad, cs_dir)
    R = st.residual(U, dt).cpu().numpy()
    assert np.abs(R - Rc.real).max() <= 1e-11 * np.abs(R).max()
    g.close()


def test_config2_scheme_gradient_against_complex_step(env):
    """The benchmarked explicit scheme (Roe, MUSCL-UNS, Barth post-limiter frozen) through 20
    SSP-RK3 steps of the Taylor-Green vortex on 6^3 x 5 tetrahedra: the adjoint gradient of
    J = sum over the centred sub-box of rho^2 V against the complex step of the numpy
    restatement on 4 seeded directions."""
    torch, ty, adjoint = env
    from typhon_gb300 import cases
    md = cases.make_mesh("tgv3d", 6)
    nci = md.ncell_int
    g = ty.Grid(md)
    g.set_spat("ROE", "MUSCL-UNS", "NONE", "BARTH", mode="exact")
    prim = cases.taylor_green(md.cell_centre)
    U0 = ty.prim_to_cons(prim[:, :nci])
    g.set_prim(prim)
    dts = [g.calc_zonetimestep(0.8)] * 20
    cc = md.cell_centre[:nci]
    L = 2 * np.pi
    box = np.all(np.abs(cc - L / 2) < L / 4, axis=1).astype(float) * md.cell_volume[:nci]
    Ut = torch.tensor(U0, device="cuda", requires_grad=True)
    J = (adjoint.rk_solve(Ut, g, "RK3-SSP", dts)[0] ** 2 * torch.tensor(box, device="cuda")).sum()
    J.backward()
    grad = Ut.grad.cpu().numpy()
    rng = np.random.default_rng(9)
    for _ in range(4):
        d = rng.standard_normal(U0.shape) * np.abs(U0).mean(axis=1, keepdims=True)
        Uc = cs.rk_run(md, U0 + 1j * 1e-30 * d, dts, adjoint.RK_TABLES["RK3-SSP"], "ROE", highres="MUSCL-UNS",
                       limiter="NONE", postlim="BARTH")
        dJ = float(np.sum(box * Uc[0] ** 2).imag / 1e-30)
        ad = float(np.sum(grad * d))
        assert abs(ad - dJ) <= 1e-8 * abs(dJ), (ad, dJ)
    g.close()


FAST_EXACT = [("HLLC", "MUSCL", "ALBADA", "NONE"), ("ROE", "MUSCL", "ALBADA", "NONE"),
              ("RUSANOV", "MUSCL", "NONE", "NONE"), ("HLLC", "MUSCL-UNS", "ALBADA", "NONE"),
              ("ROE", "MUSCL-UNS", "NONE", "BARTH"), ("HLLC", "MUSCL", "ALBADA", "SUPERBARTH")]


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("scheme,highres,limiter,postlim", FAST_EXACT)
def test_fast_second_order_vjp_equals_exact(env, dim, scheme, highres, limiter, postlim):
    """The fast mode's second-order VJP (array-of-structures records, Newton-Raphson
    reciprocals, limiter derivatives carried from the forward reconstruction) against the
    exact mode's on the same state: the same products to rounding, except where a limiter
    switch (van Albada's a b = 0, Barth's minimum) falls between the two modes' roundings of
    the same gradient, which moves single entries; hence an L2 bound and a looser max bound."""
    torch, ty, adjoint = env
    from typhon_gb300 import cases
    rng = np.random.default_rng(11)
    if dim == 2:
        md = jittered(ty, 12)
        U0 = smooth_cons(ty, md) * (1.0 + 0.05 * rng.standard_normal((1, md.ncell_int)))
    else:
        # the Taylor-Green field plus a uniform stream and per-cell noise: no face where the
        # normal velocity or a limiter argument is rounding noise (the TGV alone has such
        # faces at its symmetry points, where |vn| and van Albada's a b = 0 are kinks)
        md = cases.make_mesh("tgv3d", 4)
        nci = md.ncell_int
        prim = cases.taylor_green(md.cell_centre)[:, :nci]
        prim[2:5] += np.array([[0.3], [0.2], [0.1]]) + 0.05 * rng.standard_normal((3, nci))
        prim[:2] *= 1.0 + 0.02 * rng.standard_normal((2, nci))
        U0 = ty.prim_to_cons(prim)
    U = torch.tensor(U0, device="cuda")
    lamR = torch.tensor(rng.standard_normal(U0.shape), device="cuda")
    out = {}
    for mode in ("exact", "fast"):
        g = ty.Grid(md)
        g.set_spat(scheme, highres, limiter, postlim, mode=mode)
        st = adjoint.Stepper(g, "RK3-SSP")
        out[mode] = st.vjp(U, 1e-3, lamR).cpu().numpy()
        out[mode + "2"] = st.vjp(U, 1e-3, lamR).cpu().numpy()   # second call: tables reused
        g.close()
    assert np.array_equal(out["fast"], out["fast2"])
    diff = out["fast"] - out["exact"]
    assert np.linalg.norm(diff) <= 1e-11 * np.linalg.norm(out["exact"]), np.linalg.norm(diff)
    assert np.abs(diff).max() <= 1e-8 * np.abs(out["exact"]).max()
