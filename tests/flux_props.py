"""Helpers of the flux property tests (test infrastructure, no product code).

Typhon has no Roe flux (SOURCE/EQNS/calc_flux_inviscid.f90:48-79 stops on SCHEME = ROE), so
the Roe flux of this library is pinned by properties that any correct Roe flux has:

* consistency: F(U, U, n) equals the physical flux F_phys(U).n;
* rotational invariance: rotating both states and the normal rotates the momentum flux
  and leaves the mass and energy fluxes unchanged;
* an isolated contact discontinuity (equal pressure and velocity) is resolved exactly:
  the flux is the upwind physical flux;
* discrete conservation: on a periodic mesh the volume-weighted residuals sum to zero;
* second-order convergence on the isentropic vortex, whose exact solution is the initial
  vortex translated at the free-stream velocity.
"""
import numpy as np

GAMMA = 1.4


def physical_flux(q, nrm, gamma=GAMMA):
    """Euler flux along the unit normals: q [n][5] primitive (rho, p, u, v, w), nrm [n][3] ->
    [n][5] (mass, energy, momentum)."""
    rho, p, u = q[:, 0], q[:, 1], q[:, 2:5]
    vn = np.einsum("ij,ij->i", u, nrm)
    rhoE = p / (gamma - 1.0) + 0.5 * rho * np.einsum("ij,ij->i", u, u)
    F = np.empty_like(q)
    F[:, 0] = rho * vn
    F[:, 1] = vn * (rhoE + p)
    F[:, 2:5] = (rho * vn)[:, None] * u + p[:, None] * nrm
    return F


def random_states(rng, n, speed=1.5):
    """Primitive states with density and pressure in [0.5, 2] and velocity components in
    [-speed, speed] (sound speed about 1.2: subsonic and supersonic normal velocities)."""
    q = np.empty((n, 5))
    q[:, 0] = rng.uniform(0.5, 2.0, n)
    q[:, 1] = rng.uniform(0.5, 2.0, n)
    q[:, 2:5] = rng.uniform(-speed, speed, (n, 3))
    return q


def random_normals(rng, n):
    v = rng.standard_normal((n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def random_rotation(rng):
    """A proper rotation matrix (QR of a Gaussian matrix, sign-fixed, det +1)."""
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def rotate_prim(q, Q):
    out = q.copy()
    out[..., 2:5] = q[..., 2:5] @ Q.T
    return out


def rotate_flux(F, Q):
    out = F.copy()
    out[..., 2:5] = F[..., 2:5] @ Q.T
    return out


def vortex_exact(cases, xy, t, length=10.0, mach=0.5, gamma=GAMMA):
    """The isentropic vortex of the vortex2d case advected for time t through the periodic
    box: the initial vortex (centred in the box) translated by u_inf t, evaluated at the
    nearest periodic image."""
    uinf = mach * np.sqrt(gamma)
    xc = 0.5 * length + uinf * t
    d = xy[:, :2] - np.array([xc, 0.5 * length])
    d = d - length * np.round(d / length)          # minimum image
    pts = np.zeros((xy.shape[0], 3))
    pts[:, :2] = d + 0.5 * length
    return cases.isentropic_vortex(pts, xc=0.5 * length, yc=0.5 * length, mach=mach, gamma=gamma)


def l1_density_error(rho, rho_exact, vol):
    return float(np.sum(np.abs(rho - rho_exact) * vol) / np.sum(vol))


def rotation_z(deg):
    t = np.radians(deg)
    return np.array([[np.cos(t), -np.sin(t), 0.0], [np.sin(t), np.cos(t), 0.0], [0.0, 0.0, 1.0]])


def exact_sector(raw, right="RIGHT", left="LEFT", angle=30.0):
    """A copy of a 2D sector mesh whose `left` boundary vertices are moved onto the exact
    rotation of the matching `right` boundary vertices (mesh files store coordinates to
    single-precision-like accuracy), so that the sector is periodic to rounding."""
    import dataclasses
    bar = [(t, ie, c) for t, ie, c in raw.sections if t == 2][0]
    pos = {e: i for i, e in enumerate(bar[1])}

    def verts(fam):
        tags = [m[1] for m in raw.marks if m[0] == fam][0]
        return np.unique(bar[2][[pos[t] for t in tags]].reshape(-1)) - 1

    vr, vl = verts(right), verts(left)
    vt = raw.vtex.copy()
    rot = vt[vr] @ rotation_z(angle).T
    for i in vl:
        j = np.argmin(np.linalg.norm(rot - vt[i], axis=1))
        vt[i] = rot[j]
    return dataclasses.replace(raw, vtex=vt)


def tiled_annulus(raw, copies=12, angle=30.0, keep=("RMIN", "RMAX")):
    """The full ring of `copies` rotated copies of a periodic sector mesh (coincident vertices
    merged, so the periodic sides become interior faces); the marks in `keep` are gathered
    over all copies.  Cells of copy 0 come first, in the sector's order."""
    import dataclasses
    from scipy.spatial import cKDTree
    n = raw.vtex.shape[0]
    allv = np.concatenate([raw.vtex @ rotation_z(angle * k).T for k in range(copies)])
    tree = cKDTree(allv)
    ident = np.arange(len(allv))
    for i, j in sorted(tree.query_pairs(1e-9)):
        ident[j] = min(ident[j], ident[i])
    ident = ident[ident]                                  # first occurrence of each position
    used, newid = np.unique(ident, return_inverse=True)
    vt = allv[used]
    sections, marks = [], []
    nextel = 1
    for t, ie, c in raw.sections:
        if t == 2:
            continue
        conn = np.concatenate([newid[c - 1 + n * k] + 1 for k in range(copies)]).astype(np.int32)
        sections.append((t, np.arange(nextel, nextel + len(conn), dtype=np.int32), conn))
        nextel += len(conn)
    bar = [(t, ie, c) for t, ie, c in raw.sections if t == 2][0]
    pos = {e: i for i, e in enumerate(bar[1])}
    bconn, btag = [], {}
    for fam in keep:
        tags = [m[1] for m in raw.marks if m[0] == fam][0]
        rows = bar[2][[pos[t] for t in tags]]
        ids = []
        for k in range(copies):
            ids.extend(range(nextel + len(bconn), nextel + len(bconn) + len(rows)))
            bconn.extend((newid[rows - 1 + n * k] + 1).tolist())
        btag[fam] = np.array(ids, dtype=np.int32)
    sections.append((2, np.arange(nextel, nextel + len(bconn), dtype=np.int32), np.array(bconn, dtype=np.int32)))
    marks = [(fam, btag[fam]) for fam in keep]
    return dataclasses.replace(raw, vtex=vt, sections=sections, marks=marks)
