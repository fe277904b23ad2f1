"""Synthetic workloads: meshes and initial conditions of the benchmark configurations.

  vortex2d   2D Euler isentropic vortex (strength 5, M_inf = 0.5, gamma = 1.4) on the
             periodic [0,10]^2 box, 64x64 quads split into 8192 triangles, interior nodes
             jittered by +-10% of h (seed 1234); HLLC + MUSCL + van Albada, RK4, CFL 0.8.
  tgv3d      3D Euler Taylor-Green vortex (M = 0.1, gamma = 1.4) on the periodic
             [0,2 pi]^3 box, 64^3 hexahedra split into 5 tetrahedra (1,310,720 cells),
             interior nodes jittered by +-5% of h (seed 1234); least-squares gradients,
             MUSCL-UNS with the Barth post-limiter, Roe flux, SSP-RK3.
  ffbox3d    3D steady far-field box for the implicit solvers (FFBOX below): 48^3
             hexahedra split into 5 tetrahedra, far field on all faces, M = 0.3 at 20 degrees,
             Rusanov, a Gaussian bump relaxing to the uniform free stream.
  adjoint3d  TGV 40^3 x 5 tets, HLLC with MUSCL and van Albada, SSP-RK3, 200 steps: gradient
             of int rho^2 over a sub-box with respect to the initial state (ADJOINT3D below).
  kdif3d     3D heat conduction (KDIF3D below): 70^3 x 6 tetrahedra, lognormal
             conductivity with inclusions, two isothermal faces, implicit Euler.
All are nondimensional (rho_inf = 1).  The initial states are evaluated at cell centres.
"""
import numpy as np

from . import umesh


def isentropic_vortex(xy, xc=5.0, yc=5.0, beta=5.0, mach=0.5, gamma=1.4):
    """Primitive state (rho, p, u, v, w) of the isentropic vortex of strength beta advected at
    Mach `mach` along x (free stream rho = p = 1)."""
    x, y = xy[:, 0] - xc, xy[:, 1] - yc
    r2 = x * x + y * y
    e = np.exp(0.5 * (1.0 - r2))
    uinf = mach * np.sqrt(gamma)
    du = -beta / (2 * np.pi) * y * e
    dv = beta / (2 * np.pi) * x * e
    T = 1.0 - (gamma - 1.0) * beta * beta / (8.0 * gamma * np.pi * np.pi) * e * e
    rho = T ** (1.0 / (gamma - 1.0))
    p = rho * T
    return np.stack([rho, p, uinf + du, dv, np.zeros_like(x)])


def taylor_green(xyz, mach=0.1, gamma=1.4):
    """Primitive state of the Taylor-Green vortex (V0 = rho0 = 1, p0 = 1/(gamma M^2),
    isothermal density rho = p / p0)."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    p0 = 1.0 / (gamma * mach * mach)
    u = np.sin(x) * np.cos(y) * np.cos(z)
    v = -np.cos(x) * np.sin(y) * np.cos(z)
    p = p0 + (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2.0) / 16.0
    rho = p / p0
    return np.stack([rho, p, u, v, np.zeros_like(x)])


def perturbed_freestream(xyz, ff, centre, amp=0.2, width=1.0):
    """The free stream ff = (rho, p, u, v, w) with a Gaussian bump of density, pressure and
    velocity around `centre`."""
    r2 = ((xyz - np.asarray(centre)) ** 2).sum(1)
    b = amp * np.exp(-r2 / width)
    return np.stack([ff[0] * (1 + b), ff[1] * (1 + b), ff[2] + 0.5 * b, ff[3] - 0.5 * b, ff[4] + 0.25 * b])


_ANG = np.deg2rad(20.0)
# 3D steady far-field box: free stream M = 0.3 at 20 degrees through far-field boundaries on all
# six faces of the [0, 2 pi]^3 tetrahedral box, a Gaussian bump in the initial state; the steady
# state is the uniform free stream.  Rusanov flux with its own Jacobian (Newton-consistent).
FFBOX = dict(dim=3, n=48, length=2 * np.pi, jitter=0.05, seed=1234, scheme="RUSANOV", highres="NONE",
             limiter="NONE", postlim="NONE",
             freestream=(1.0, 1.0 / 1.4, 0.3 * np.cos(_ANG), 0.3 * np.sin(_ANG) * 0.6, 0.3 * np.sin(_ANG) * 0.8),
             cfl0=10.0, cfl_max=25.0, nkrylov=30, max_it=2, inv_res=1e-2, target=1e-10, max_steps=1500)


# config 3: laminar flat plate, M = 0.3, Re_L = 1e4 on the plate's unit length, air at 288 K
# (Sutherland), adiabatic no-slip wall, far field at the inlet, outlet and top, symmetry
# upstream of the plate and on the span sides; 2 nx nz 50 prisms + 6 nx nz 25 tetrahedra
# (nx = 200, nz = 20: 400,000 + 600,000 cells).  First-order Rusanov with its own Jacobian
# and the cell-average viscous flux (Typhon's scalar viscous Jacobian); backward Euler with
# local time steps, CFL 10 ramped by 1.5 per step to cfl_max, row-scaled FGMRES(nkrylov) x
# max_it to INV_RES.  Newton with exact solves converges at any CFL; the cap is where ~600
# block-Jacobi FGMRES iterations still solve the system (CFL 500 - 1000 on this mesh), and
# short restarts keep the FP64 Gram sweeps cheap.
_T_FP = 288.0
_A_FP = float(np.sqrt(1.4 * 287.14 * _T_FP))
_MU_FP = 1.68e-5 * (_T_FP / 273.0) ** 1.5 * (273.0 + 110.5) / (_T_FP + 110.5)
_RHO_FP = 1e4 * _MU_FP / (0.3 * _A_FP)
FLATPLATE = dict(nx=200, nz=20, scheme="RUSANOV", rgas=287.14, prandtl=0.72,
                 freestream=(_RHO_FP, _RHO_FP * 287.14 * _T_FP, 0.3 * _A_FP, 0.0, 0.0),
                 cfl0=10.0, cfl_max=500.0, nkrylov=15, max_it=40, inv_res=0.05, target=1e-10, max_steps=20000)


def make_flatplate(nx=None, nz=None):
    """Preprocessed flat-plate mesh of FLATPLATE (native preprocessing)."""
    w = FLATPLATE
    nx, nz = nx or w["nx"], nz or w["nz"]
    raw = umesh.gen_flatplate(nx=nx, nz=nz, width=0.01 * nz)
    return umesh.preprocess(raw, 3, umesh.flatplate_bcs())


def make_ffbox(n=None):
    """Preprocessed far-field tetrahedral box of FFBOX (native preprocessing)."""
    w = FFBOX
    n = n or w["n"]
    raw = umesh.gen_tet_box(n, w["length"], jitter=w["jitter"], seed=w["seed"])
    bcs = [(f, umesh.BC_FARFIELD, "", (0.0, 0.0, 0.0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX", "KMIN", "KMAX")]
    return umesh.preprocess(raw, 3, bcs)


# 3D heat conduction: unit cube of 70^3 hexahedra x 6 tetrahedra (2,058,000 cells), seeded
# lognormal conductivity (sigma = 1) with 8 random spherical inclusions of radius 0.1 at 100x,
# T = 0 / 1 on the x faces, adiabatic elsewhere, backward Euler dt = 1e-3 for 50 steps.
KDIF3D = dict(n=70, sigma=1.0, inclusions=8, radius=0.1, contrast=100.0, seed=1234, dt=1e-3, steps=50,
              heat_capacity=1.0, tol=1e-12)


def make_kdif3d(n=None):
    """Mesh (MeshDesc), per-cell conductivity, boundary kinds and values of KDIF3D."""
    w = KDIF3D
    n = n or w["n"]
    raw = umesh.gen_kuhn_box(n, 1.0)
    bcs = [(f, umesh.BC_WALL, "", (0.0, 0.0, 0.0)) for f in ("IMIN", "IMAX", "JMIN", "JMAX", "KMIN", "KMAX")]
    md = umesh.preprocess(raw, 3, bcs)
    rng = np.random.default_rng(w["seed"])
    nci = md.ncell_int
    k = np.exp(w["sigma"] * rng.standard_normal(nci))
    cc = md.cell_centre[:nci]
    for c in rng.uniform(w["radius"], 1.0 - w["radius"], size=(w["inclusions"], 3)):
        k[((cc - c) ** 2).sum(1) < w["radius"] ** 2] *= w["contrast"]
    kind = np.zeros(md.nface, np.int32)
    val = np.zeros(md.nface)
    fc = md.face_centre
    b = np.arange(md.nface_int, md.nface)
    kind[b] = 2                                       # imposed flux 0: adiabatic
    x0 = b[np.abs(fc[b, 0]) < 1e-12]
    x1 = b[np.abs(fc[b, 0] - 1.0) < 1e-12]
    kind[x0], val[x0] = 1, 0.0                        # isothermal T = 0
    kind[x1], val[x1] = 1, 1.0                        # isothermal T = 1
    return md, k, kind, val


# 3D Euler adjoint: the Taylor-Green vortex on 40^3 x 5 tetrahedra (320,000 cells), first-order
# Roe residual (the adjoint covers first-order residuals), SSP-RK3 at a fixed time step,
# J = integral of rho^2 over the centred sub-box [pi/2, 3 pi/2]^3 at the final time; its
# gradient with respect to the initial state by the adjoint with 20 stored states, and 16
# seeded directional derivatives of it checked by central finite differences.
ADJOINT3D = dict(n=40, steps=200, snaps=20, directions=16, scheme="HLLC", highres="MUSCL", limiter="ALBADA",
                 rk="RK3-SSP", cfl=0.8, seed=1234)


WORKLOADS = {
    "vortex2d": dict(dim=2, n=64, length=10.0, jitter=0.10, seed=1234, scheme="HLLC", highres="MUSCL",
                     limiter="ALBADA", postlim="NONE", rk="RK4", cfl=0.8, steps=200),
    "tgv3d": dict(dim=3, n=64, length=2 * np.pi, jitter=0.05, seed=1234, scheme="ROE", highres="MUSCL-UNS",
                  limiter="NONE", postlim="BARTH", rk="RK3-SSP", cfl=0.8, steps=500),
}


def shuffle_cells(raw, seed=1):
    """The same mesh with the element rows of each cell section in a random order (seeded):
    a stand-in for a mesh file whose numbering scatters neighbouring cells."""
    rng = np.random.default_rng(seed)
    dmax = max(umesh.DIM[t] for t, _, _ in raw.sections)
    secs = [(t, ie, conn[rng.permutation(len(ie))] if umesh.DIM[t] == dmax else conn) for t, ie, conn in raw.sections]
    return umesh.RawMesh(vtex=raw.vtex, sections=secs, marks=list(raw.marks))


def make_raw(name, n=None, cell_order="given"):
    """Element mesh of a workload.  cell_order: "given" (the generator's numbering),
    "shuffled" (rows of the cell section permuted at random), "shuffled-rcm" (shuffled,
    then renumbered in reverse Cuthill-McKee order)."""
    w = WORKLOADS[name]
    n = n or w["n"]
    if w["dim"] == 2:
        raw = umesh.gen_grid2d(n, n, w["length"], w["length"], "tri", jitter=w["jitter"], seed=w["seed"])
    else:
        raw = umesh.gen_tet_box(n, w["length"], jitter=w["jitter"], seed=w["seed"])
    if cell_order == "given":
        return raw
    raw = shuffle_cells(raw)
    if cell_order == "shuffled":
        return raw
    if cell_order == "shuffled-rcm":
        return umesh.reorder_rcm(raw, w["dim"], umesh.periodic_box_bcs((w["length"],) * w["dim"]))
    raise ValueError(f"cell_order {cell_order!r}")


def make_mesh(name, n=None, cell_order="given"):
    """Preprocessed mesh of a workload (native preprocessing)."""
    w = WORKLOADS[name]
    raw = make_raw(name, n, cell_order)
    return umesh.preprocess(raw, w["dim"], umesh.periodic_box_bcs((w["length"],) * w["dim"]))


def initial_prim(name, centres):
    if name == "vortex2d":
        return isentropic_vortex(centres)
    return taylor_green(centres)
