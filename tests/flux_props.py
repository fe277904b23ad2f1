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
