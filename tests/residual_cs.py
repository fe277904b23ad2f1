"""Complex-step reference of the residual (test infrastructure).

A numpy restatement of the residual R = dt/V sum(+-F S) (Rusanov, HLLC and Roe fluxes; first
order with periodic and symmetry boundaries, or least-squares gradients with MUSCL / MUSCL-UNS,
van Albada and the frozen Barth post-limiter on periodic meshes) written so that it is analytic
in the state: the
absolute value is z sign(Re z), max/min compare real parts, the square root is the complex
one.  Evaluated at U + i h d it gives dR/dU d to machine precision (complex step), and with
the Runge-Kutta tables of typhon_gb300.adjoint the derivative of a whole explicit run.
"""
import numpy as np


def cabs(z):
    return z * np.sign(z.real)


def cmax(a, b):
    return np.where(a.real >= b.real, a, b)


def prim(U, g):
    rho = U[0]
    u, v, w = U[2] / rho, U[3] / rho, U[4] / rho
    p = (g - 1.0) * (U[1] - 0.5 * rho * (u * u + v * v + w * w))
    return np.stack([rho, p, u, v, w])


def rusanov(L, R, n, g):
    ig1 = 1.0 / (g - 1.0)
    vnl = L[2] * n[0] + L[3] * n[1] + L[4] * n[2]
    vnr = R[2] * n[0] + R[3] * n[1] + R[4] * n[2]
    al, ar = np.sqrt(g * L[1] / L[0]), np.sqrt(g * R[1] / R[0])
    ray = cmax(cabs(vnl) + al, cabs(vnr) + ar)
    rel = ig1 * L[1] + 0.5 * L[0] * (L[2] ** 2 + L[3] ** 2 + L[4] ** 2)
    rer = ig1 * R[1] + 0.5 * R[0] * (R[2] ** 2 + R[3] ** 2 + R[4] ** 2)
    a, b = (vnl + ray) * L[0], (vnr - ray) * R[0]
    F = [0.5 * (a + b), 0.5 * ((vnl + ray) * rel + (vnr - ray) * rer + vnl * L[1] + vnr * R[1])]
    for k in range(3):
        F.append(0.5 * ((a * L[2 + k] + b * R[2 + k]) + (L[1] + R[1]) * n[k]))
    return np.stack(F)


def cmin(a, b):
    return np.where(b.real < a.real, b, a)


def hllc(L, R, n, g):
    """HLLC with Roe-averaged wave-speed estimates (SOURCE/VALE/calc_flux_hllc.f90)."""
    ig1, gig1 = 1.0 / (g - 1.0), g / (g - 1.0)
    t1 = np.sqrt(R[0] / L[0])
    roe_rho = L[0] * t1
    kl = 1.0 / (1.0 + t1)
    kr = t1 * kl
    ru = [kl * L[2 + k] + kr * R[2 + k] for k in range(3)]
    sqL = L[2] ** 2 + L[3] ** 2 + L[4] ** 2
    sqR = R[2] ** 2 + R[3] ** 2 + R[4] ** 2
    h = kl * (gig1 * L[1] / L[0] + 0.5 * sqL) + kr * (gig1 * R[1] / R[0] + 0.5 * sqR)
    roe_p = (h - 0.5 * (ru[0] ** 2 + ru[1] ** 2 + ru[2] ** 2)) * roe_rho / gig1
    vnl = L[2] * n[0] + L[3] * n[1] + L[4] * n[2]
    vnr = R[2] * n[0] + R[3] * n[1] + R[4] * n[2]
    al, ar = np.sqrt(g * L[1] / L[0]), np.sqrt(g * R[1] / R[0])
    vm = ru[0] * n[0] + ru[1] * n[1] + ru[2] * n[2]
    am = np.sqrt(g * roe_p / roe_rho)
    rel = ig1 * L[1] + 0.5 * L[0] * sqL
    rer = ig1 * R[1] + 0.5 * R[0] * sqR
    sl = cmin(vnl - al, vm - am)
    sr = cmax(vm + am, vnr + ar)

    def side_flux(Q, vq, re):
        m0 = vq * Q[0]
        return np.stack([m0, vq * (re + Q[1])] + [m0 * Q[2 + k] + Q[1] * n[k] for k in range(3)])

    rqL, rqR = L[0] * (sl - vnl), R[0] * (sr - vnr)
    Sst = (rqR * vnr - rqL * vnl - R[1] + L[1]) / (rqR - rqL)
    left = Sst.real >= 0.0

    def star_flux(Q, s, vq, rq, re):
        iks = 1.0 / (s - Sst)
        pst = Q[1] - rq * (vq - Sst)
        dp = pst - Q[1]
        rest = iks * (re * (s - vq) - Q[1] * vq + pst * Sst)
        return np.stack([Sst * (rq * iks), Sst * (rest + pst)] +
                        [Sst * (iks * (rq * Q[2 + k] + dp * n[k])) + pst * n[k] for k in range(3)])

    Fs = np.where(left, star_flux(L, sl, vnl, rqL, rel), star_flux(R, sr, vnr, rqR, rer))
    F = np.where(sr.real <= 0.0, side_flux(R, vnr, rer), Fs)
    return np.where(sl.real >= 0.0, side_flux(L, vnl, rel), F)


def roe(L, R, n, g, eps=0.1):
    ig1, gig1 = 1.0 / (g - 1.0), g / (g - 1.0)
    t1 = np.sqrt(R[0] / L[0])
    rroe = L[0] * t1
    kl = 1.0 / (1.0 + t1)
    kr = t1 * kl
    u = [kl * L[2 + k] + kr * R[2 + k] for k in range(3)]
    sqL = L[2] ** 2 + L[3] ** 2 + L[4] ** 2
    sqR = R[2] ** 2 + R[3] ** 2 + R[4] ** 2
    hroe = kl * (gig1 * L[1] / L[0] + 0.5 * sqL) + kr * (gig1 * R[1] / R[0] + 0.5 * sqR)
    q2 = u[0] ** 2 + u[1] ** 2 + u[2] ** 2
    a2 = (g - 1.0) * (hroe - 0.5 * q2)
    a = np.sqrt(a2)
    vn = u[0] * n[0] + u[1] * n[1] + u[2] * n[2]
    vnl = L[2] * n[0] + L[3] * n[1] + L[4] * n[2]
    vnr = R[2] * n[0] + R[3] * n[1] + R[4] * n[2]
    rel = ig1 * L[1] + 0.5 * L[0] * sqL
    rer = ig1 * R[1] + 0.5 * R[0] * sqR
    drho, dp, dvn = R[0] - L[0], R[1] - L[1], vnr - vnl
    du = [R[2 + k] - L[2 + k] for k in range(3)]
    al1 = (dp - rroe * a * dvn) / (2.0 * a2)
    al5 = (dp + rroe * a * dvn) / (2.0 * a2)
    al2 = drho - dp / a2
    dut = [du[k] - dvn * n[k] for k in range(3)]
    l1, l5, l2 = cabs(vn - a), cabs(vn + a), cabs(vn)
    delta = eps * a
    l1 = np.where(l1.real < delta.real, (l1 * l1 + delta * delta) / (2.0 * delta), l1)
    l5 = np.where(l5.real < delta.real, (l5 * l5 + delta * delta) / (2.0 * delta), l5)
    w1, w2, w5, ws = l1 * al1, l2 * al2, l5 * al5, l2 * rroe
    dm = [w1 * (u[k] - a * n[k]) + w2 * u[k] + w5 * (u[k] + a * n[k]) + ws * dut[k] for k in range(3)]
    de = w1 * (hroe - a * vn) + w2 * (0.5 * q2) + w5 * (hroe + a * vn) + ws * (
        (u[0] * du[0] + u[1] * du[1] + u[2] * du[2]) - vn * dvn)
    ml, mr = vnl * L[0], vnr * R[0]
    F = [0.5 * (ml + mr - (w1 + w2 + w5)), 0.5 * (vnl * (rel + L[1]) + vnr * (rer + R[1]) - de)]
    for k in range(3):
        F.append(0.5 * ((ml * L[2 + k] + L[1] * n[k]) + (mr * R[2 + k] + R[1] * n[k]) - dm[k]))
    return np.stack(F)


def _ghost_source(md):
    """Cell whose state each cell carries: itself, or for a periodic ghost the partner's cell."""
    src = np.arange(md.ncell)
    b = np.arange(md.nface_int, md.nface)
    per = b[md.face_bc[b] == 1]
    src[md.fc2[per]] = md.fc1[md.face_partner[per] - 1]
    return src


def lsq_weights(md):
    """w[side, f] = A_c^-1 d_f for the cell c on that side of face f (precalc_grad_lsq.f90: A_c
    = sum of d d^T over the cell's faces, d = C(fc2) - C(fc1); one added to A_zz in 2D)."""
    nci, nf = md.ncell_int, md.nface
    d = md.cell_centre[md.fc2] - md.cell_centre[md.fc1]
    A = np.zeros((nci, 3, 3))
    dd = d[:, :, None] * d[:, None, :]
    np.add.at(A, md.fc1, dd)
    inner = np.arange(md.nface_int)
    np.add.at(A, md.fc2[inner], dd[inner])
    if md.dim == 2:
        A[:, 2, 2] += 1.0
    Ainv = np.linalg.inv(A)
    w = np.zeros((2, nf, 3))
    w[0] = np.einsum("fij,fj->fi", Ainv[md.fc1], d)
    w[1, inner] = np.einsum("fij,fj->fi", Ainv[md.fc2[inner]], d[inner])
    return w


def gradient(md, P, w):
    """G [5, ncell_int, 3] = sum over the cell's faces of w (P(fc2) - P(fc1))."""
    nci = md.ncell_int
    dP = P[:, md.fc2] - P[:, md.fc1]                        # [5, nf] (ghosts carry their source)
    G = np.zeros((5, nci, 3), dtype=P.dtype)
    inner = np.arange(md.nface_int)
    for k in range(3):
        np.add.at(G[:, :, k].T, md.fc1, (dP * w[0, :, k]).T)
        np.add.at(G[:, :, k].T, md.fc2[inner], (dP[:, inner] * w[1, inner, k]).T)
    return G


def muscl(md, P, G, faces, side, limiter, highres="MUSCL"):
    """MUSCL state of one side of `faces`: q_c + G_c.CF + sg (u.CF), sg = phi(a, LR) - g with
    van Albada's phi (or LR - g without limiter), a = 2g - LR for HIGHRES = MUSCL
    (tvdgradstr) and a = g for MUSCL-UNS (tvdgraduns)."""
    fc1, fc2 = md.fc1[faces], md.fc2[faces]
    c = fc2 if side else fc1
    CL, CR = md.cell_centre[fc1], md.cell_centre[fc2]
    dv = CR - CL
    dLR = np.sqrt(np.sum(dv * dv, axis=1))
    u = dv / dLR[:, None]
    CF = md.face_centre[faces] - (CR if side else CL)
    uc = np.sum(u * CF, axis=1)
    LR = (P[:, fc2] - P[:, fc1]) / dLR
    Gc = G[:, c, :]
    g = np.einsum("vfk,fk->vf", Gc, u)
    if limiter == "ALBADA":
        a, b = (g if highres == "MUSCL-UNS" else 2.0 * g - LR), LR
        pos = (a.real * b.real) > 0.0
        den = np.where(pos, a * a + b * b, 1.0)
        phi = np.where(pos, a * b * (a + b) / den, 0.0)
        sg = phi - g
    else:
        sg = LR - g
    return P[:, c] + np.einsum("vfk,fk->vf", Gc, CF) + sg * uc


def barth_ratios(md, P, QL, QR, klim=0.5):
    """Typhon's face-ratio post-limiter (postlimit_barth.f90:42-223) from the real parts:
    r[group, c] = min(1, min over the cell's faces and the group's variables of
    max(klim (q_nb - q_c) / (q_face - q_c), 0)), groups rho, p and the velocity vector; a face
    whose increment is exactly zero imposes no constraint.  The ratios are real: a complex
    step through the limited states differentiates the limiter frozen at them."""
    nci, nfi = md.ncell_int, md.nface_int
    Pr, QLr, QRr = P.real, QL.real, QR.real
    r = np.ones((3, nci))
    grp = [0, 1, 2, 2, 2]
    inner = np.arange(nfi)
    for cells, nb, q, sel in ((md.fc1, md.fc2, QLr, np.arange(md.nface)),
                              (md.fc2[inner], md.fc1[inner], QRr[:, inner], inner)):
        c, n = cells, nb
        for v in range(5):
            den = q[v] - Pr[v, c]
            dq = Pr[v, n] - Pr[v, c]
            ok = den != 0.0
            t = np.full(den.shape, np.inf)
            t[ok] = np.maximum(klim * (dq[ok] / den[ok]), 0.0)
            np.minimum.at(r[grp[v]], c, t)
    return r


def residual(md, U, dt, scheme="RUSANOV", g=1.4, highres="NONE", limiter="NONE", postlim="NONE"):
    """R [5, ncell_int] of the residual at U [5, ncell_int] (real or complex): first order, or
    least-squares gradients and MUSCL / MUSCL-UNS with no limiter or van Albada, optionally
    Typhon's Barth post-limiter with its ratios frozen (periodic boundaries)."""
    nci, nf, nfi = md.ncell_int, md.nface, md.nface_int
    fc1, fc2 = md.fc1, md.fc2
    P = prim(U, g)
    if highres != "NONE":
        P = P[:, _ghost_source(md)]
        G = gradient(md, P, lsq_weights(md))
        allf = np.arange(nf)
        QL = muscl(md, P, G, allf, 0, limiter, highres)
        QR = np.empty_like(QL)
        inner = np.arange(nfi)
        QR[:, inner] = muscl(md, P, G, inner, 1, limiter, highres)
        b = np.arange(nfi, nf)
        if postlim != "NONE":
            r = barth_ratios(md, P, QL, QR, 0.5 if postlim == "BARTH" else 1.0)
            grp = [0, 1, 2, 2, 2]
            for v in range(5):
                QL[v] = P[v, fc1] + r[grp[v], fc1] * (QL[v] - P[v, fc1])
                QR[v, inner] = P[v, fc2[inner]] + r[grp[v], fc2[inner]] * (QR[v, inner] - P[v, fc2[inner]])
            QR[:, b] = QL[:, md.face_partner[b] - 1]
        else:
            QR[:, b] = muscl(md, P, G, md.face_partner[b] - 1, 0, limiter, highres)
        n = md.face_normal.T
        F = {"RUSANOV": rusanov, "HLLC": hllc, "ROE": roe}[scheme](QL, QR, n, g) * md.face_surface
        R = np.zeros((5, nci), dtype=U.dtype)
        np.subtract.at(R.T, fc1, F.T)
        np.add.at(R.T, fc2[inner], F[:, inner].T)
        return dt / md.cell_volume[:nci] * R
    QL = P[:, fc1]
    right = np.where(np.arange(nf) < nfi, fc2, 0)
    QR = P[:, np.minimum(right, nci - 1)].copy()
    n = md.face_normal.T
    b = np.arange(nfi, nf)
    per = b[md.face_bc[b] == 1]
    QR[:, per] = P[:, fc1[md.face_partner[per] - 1]]
    sym = b[md.face_bc[b] == 2]
    dn = 2.0 * (QL[2, sym] * n[0, sym] + QL[3, sym] * n[1, sym] + QL[4, sym] * n[2, sym])
    QR[:, sym] = QL[:, sym]
    for k in range(3):
        QR[2 + k, sym] = QL[2 + k, sym] - dn * n[k, sym]
    F = {"RUSANOV": rusanov, "HLLC": hllc, "ROE": roe}[scheme](QL, QR, n, g) * md.face_surface
    R = np.zeros((5, nci), dtype=U.dtype)
    np.subtract.at(R.T, fc1, F.T)
    inner = np.arange(nfi)
    np.add.at(R.T, fc2[inner], F[:, inner].T)
    return dt / md.cell_volume[:nci] * R


def rk_run(md, U0, dts, table, scheme="RUSANOV", highres="NONE", limiter="NONE", postlim="NONE"):
    U = U0
    for dt in dts:
        Rs = []
        for k in range(len(table)):
            Uk = U.copy()
            for s in range(k):
                if table[k - 1][s] != 0.0:
                    Uk = Uk + table[k - 1][s] * Rs[s]
            Rs.append(residual(md, Uk, dt, scheme, highres=highres, limiter=limiter, postlim=postlim))
        for s, c in enumerate(table[-1]):
            if c != 0.0:
                U = U + c * Rs[s]
    return U


def box_functional_derivative(md, U0, d, dts, table, box, scheme, highres="NONE", limiter="NONE", postlim="NONE",
                              h=1e-30):
    """Complex-step derivative along d of J(U0) = sum(box * rho^2) after an explicit run (the
    reference of the adjoint's directional derivatives)."""
    Uc = rk_run(md, U0 + 1j * h * d, dts, table, scheme, highres=highres, limiter=limiter, postlim=postlim)
    return float(np.sum(box * Uc[0] ** 2).imag / h)
