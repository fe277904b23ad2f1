// Typhon CPU oracle, heat conduction (KDIF) — TEST INFRASTRUCTURE ONLY.
//
// Restates the cell-centred conduction residual of Typhon's KDIF solver and its implicit
// (backward Euler) step, for checking the GPU library:
//   face flux            SOURCE/EQKDIF/calc_kdif_flux.f90:76-177 (compact, cell-average and
//                        full face gradients, theta = 1) and its Jacobian :169-175
//   boundary conditions  setboco_kdif_isoth.f90 (ghost temperature = wall temperature),
//                        setboco_kdif_flux.f90 + kdif_bocoflux.f90 (imposed flux, ghost =
//                        inside; Jacobian J_L += J_R, J_R = 0)
//   residual             flux_to_res.f90 (colour order, dt/V), U = Cp T (calc_varcons_kdif)
//   implicit matrix      build_implicit_dlu (scalar form of build_implicit_bdlu.f90)
// New, with no Typhon counterpart: a conductivity per cell (Typhon's material is uniform or
// a law of T), whose face value is the distance-weighted harmonic mean of the two cells'
// (the cells' common value when they are equal); and conjugate gradients on the
// symmetrised system diag(V/dt) A, which is symmetric positive definite (Typhon offers
// CGS, BiCG and GMRES).
#include <cmath>
#include <cstring>
#include <limits>
#include <algorithm>
#include <vector>

#include "oracle.hpp"

namespace ory {

void KdifSolver::init(const UMesh* mesh, int flux_scheme, double heat_capacity, const double* kc, const int* kind,
                      const double* value) {
  m = mesh;
  scheme = flux_scheme;
  cp = heat_capacity;
  const int nc = m->ncell, nci = m->ncell_int, nf = m->nface;
  kcell.assign(nc, 0.0);
  for (int c = 0; c < nci; ++c) kcell[c] = kc[c];
  fkind.assign(nf, 0);
  fval.assign(nf, 0.0);
  for (int f = m->nface_int; f < nf; ++f) {
    fkind[f] = kind[f];
    fval[f] = value[f];
    kcell[m->fc2[f]] = kcell[m->fc1[f]];
  }
  for (auto& b : m->bocos)
    if (b.kind == BC_PERIODIC)
      for (size_t k = 0; k < b.iface.size(); ++k) {
        fkind[b.iface[k]] = KBC_PERIODIC;
        kcell[m->fc2[b.iface[k]]] = kcell[m->fc1[b.partner_face[k]]];
      }
  T.assign(nc, 0.0);
  grad.assign(3 * (size_t)nc, 0.0);
  flux.assign(nf, 0.0);
  jac.assign(nf, 0.0);
  residu.assign(nc, 0.0);
  lsq.m = m;
  SpatParams sp;
  sp.gradmeth = GRAD_LSQ;
  lsq.init(m, sp, RK4, 1.0);
}

// ghost temperatures (calcboco_kdif.f90 cell-state mode)
void KdifSolver::ghosts() {
  for (auto& b : m->bocos)
    for (size_t k = 0; k < b.iface.size(); ++k) {
      const int f = b.iface[k], g = m->fc2[f];
      if (b.kind == BC_PERIODIC) T[g] = T[m->fc1[b.partner_face[k]]];
      else if (fkind[f] == KBC_ISOTHERMAL) T[g] = fval[f];
      else T[g] = T[m->fc1[f]];
    }
}

// calc_gradient on T: the least-squares gradient of the NS path applied to one scalar
void KdifSolver::gradient() {
  const int nc = m->ncell;
  std::fill(lsq.prim.begin(), lsq.prim.end(), 0.0);
  for (int c = 0; c < nc; ++c) lsq.prim[c] = T[c];
  lsq.calc_gradient();
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < m->ncell_int; ++c) grad[k * (size_t)nc + c] = lsq.grad[k * (size_t)nc + c];
}

double KdifSolver::face_k(int f, double dHL, double dHR) const {
  const double kl = kcell[m->fc1[f]], kr = kcell[m->fc2[f]];
  if (kl == kr) return kl;
  return 1.0 / (dHL / kl + dHR / kr);
}

// calc_kdif_flux (per unit surface) + kdif_bocoflux, then times S (flux_to_res)
void KdifSolver::fluxes() {
  const int nc = m->ncell, nf = m->nface;
  const double theta = 1.0;
  for (int f = 0; f < nf; ++f) {
    const int icl = m->fc1[f], icr = m->fc2[f];
    const V3 F = m->fcentre[f], CL = m->ccentre[icl], CR = m->ccentre[icr], n = m->fnormal[f];
    double dHL = vabs(F - CL), dHR = vabs(F - CR);
    const double id = 1.0 / (dHL + dHR);
    dHL = id * dHL;
    dHR = id * dHR;
    const V3 vLR = CR - CL;
    const double dLR = vabs(vLR);
    const double kH = face_k(f, dHL, dHR);
    const V3 gL = v3(grad[icl], grad[nc + icl], grad[2 * (size_t)nc + icl]);
    const V3 gR = v3(grad[icr], grad[nc + icr], grad[2 * (size_t)nc + icr]);
    double Fl;
    if (scheme == KDIF_COMPACT) {
      Fl = -kH * (T[icr] - T[icl]) * dot(vLR, n) / (dLR * dLR);
    } else if (scheme == KDIF_CELLAVG) {
      Fl = -kH * dot(dHL * gR + dHR * gL, n);
    } else {
      const double pscal = dot(vLR, n) / (dLR * dLR);
      const double Fcomp = pscal * (T[icr] - T[icl]);
      const V3 vi = n - (theta * pscal) * vLR;
      const double Favg = dot(dHL * gR + dHR * gL, vi);
      Fl = -kH * (theta * Fcomp + Favg);
    }
    double jR = -kH * dot(vLR, n) / (cp * (dLR * dLR));
    if (fkind[f] == KBC_FLUX) {  // imposed flux entering the domain, reversed (setboco_kdif_flux.f90)
      Fl = -fval[f];
      jR = 0.0;                   // J_L + J_R = 0 and J_R = 0 (kdif_bocoflux.f90)
    }
    flux[f] = m->fsurf[f] * Fl;
    jac[f] = m->fsurf[f] * jR;
  }
}

void KdifSolver::rhs(double dt) {
  const int nci = m->ncell_int;
  ghosts();
  if (scheme != KDIF_COMPACT) gradient();
  fluxes();
  std::fill(residu.begin(), residu.end(), 0.0);
  for (auto& col : m->colors)
    for (int f : col) {
      residu[m->fc1[f]] = residu[m->fc1[f]] - flux[f];
      residu[m->fc2[f]] = residu[m->fc2[f]] + flux[f];
    }
  balance.assign(residu.begin(), residu.begin() + nci);
  for (int c = 0; c < nci; ++c) residu[c] = dt / m->cvol[c] * residu[c];
}

// symmetrised implicit system diag(V/dt) A dU = sum(+-F S): diagonal V/dt - sum_f J_R S over
// the cell's faces in face order, off-diagonal J_R S; U = Cp T, so T += dU / Cp
void KdifSolver::assemble(double dt) {
  const int nci = m->ncell_int, nf = m->nface;
  diag.assign(nci, 0.0);
  for (int c = 0; c < nci; ++c) diag[c] = m->cvol[c] / dt;
  for (int f = 0; f < nf; ++f) {
    const int c1 = m->fc1[f], c2 = m->fc2[f];
    diag[c1] = diag[c1] - jac[f];
    if (f < m->nface_int) diag[c2] = diag[c2] - jac[f];
  }
}

void KdifSolver::matvec(const double* x, double* y) const {
  const int nci = m->ncell_int;
  for (int c = 0; c < nci; ++c) y[c] = diag[c] * x[c];
  for (int f = 0; f < m->nface_int; ++f) {
    const int c1 = m->fc1[f], c2 = m->fc2[f];
    y[c1] = y[c1] + jac[f] * x[c2];
    y[c2] = y[c2] + jac[f] * x[c1];
  }
}

// conjugate gradients with Jacobi preconditioning, relative residual tol
int KdifSolver::cg(const std::vector<double>& b, std::vector<double>& x, double tol, int max_it, double* rel) {
  const int n = m->ncell_int;
  x.assign(n, 0.0);
  std::vector<double> r(b), z(n), p(n), q(n);
  auto dotv = [&](const std::vector<double>& a, const std::vector<double>& c) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * c[i];
    return s;
  };
  const double bn = std::sqrt(dotv(b, b));
  if (!(bn > 0.0)) { *rel = 0.0; return 0; }
  for (int i = 0; i < n; ++i) z[i] = r[i] / diag[i];
  p = z;
  double rz = dotv(r, z);
  int it = 0;
  *rel = 1.0;
  for (it = 1; it <= max_it; ++it) {
    matvec(p.data(), q.data());
    const double alpha = rz / dotv(p, q);
    for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    *rel = std::sqrt(dotv(r, r)) / bn;
    if (*rel < tol) break;
    for (int i = 0; i < n; ++i) z[i] = r[i] / diag[i];
    const double rz2 = dotv(r, z);
    const double beta = rz2 / rz;
    rz = rz2;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  return it;
}

int KdifSolver::implicit_step(double dt, double tol, int max_it, double* rel) {
  rhs(dt);
  assemble(dt);
  std::vector<double> x;
  int it = cg(balance, x, tol, max_it, rel);
  for (int c = 0; c < m->ncell_int; ++c) T[c] = T[c] + x[c] / cp;
  return it;
}

// calc_kdif_timestep.f90:38-62 (linear material), then the global minimum over the cells
// (calc_zonetimestep.f90, stability condition)
double KdifSolver::fourier_dt(double fourier, double conduct) const {
  const int nci = m->ncell_int;
  std::vector<double> d(nci, 0.0);
  for (int f = 0; f < m->nface_int; ++f) {
    const double s2 = m->fsurf[f] * m->fsurf[f];
    d[m->fc1[f]] = d[m->fc1[f]] + s2;
    d[m->fc2[f]] = d[m->fc2[f]] + s2;
  }
  for (int f = m->nface_int; f < m->nface; ++f) d[m->fc1[f]] = d[m->fc1[f]] + m->fsurf[f] * m->fsurf[f];
  double dt = std::numeric_limits<double>::max();
  for (int c = 0; c < nci; ++c) {
    const double v = m->cvol[c];
    double x = 2.0 * fourier * (v * v) / d[c];
    x = x * cp / conduct;
    dt = std::min(dt, x);
  }
  return dt;
}

// init_implicit_dlu.f90 (unit diagonal) + build_implicit_dlu.f90:44-66 with J_L = -J_R,
// both times S (flux_to_res.f90:76-80); rows and columns over all cells, ghosts included
void KdifSolver::typhon_dlu(double dt) {
  const int nc = m->ncell, nci = m->ncell_int, nf = m->nface, nfi = m->nface_int;
  dlu_diag.assign(nc, 0.0);
  dlu_upper.assign(nf, 0.0);
  dlu_lower.assign(nf, 0.0);
  for (int c = 0; c < nci; ++c) dlu_diag[c] = 1.0;
  for (int f = 0; f < nfi; ++f) {
    const int c1 = m->fc1[f], c2 = m->fc2[f];
    const double jR = jac[f], jL = -jac[f];
    dlu_diag[c1] = dlu_diag[c1] + jL * dt / m->cvol[c1];
    dlu_upper[f] = jR * dt / m->cvol[c1];
    dlu_diag[c2] = dlu_diag[c2] - jR * dt / m->cvol[c2];
    dlu_lower[f] = -(jL * dt / m->cvol[c2]);
  }
  for (int f = nfi; f < nf; ++f) {
    const int c1 = m->fc1[f], c2 = m->fc2[f];
    const double jR = jac[f], jL = -jac[f];
    dlu_diag[c1] = dlu_diag[c1] + jL * dt / m->cvol[c1];
    dlu_upper[f] = jR * dt / m->cvol[c1];
    dlu_diag[c2] = 1.0;
    dlu_lower[f] = 0.0;
  }
}

// SPMAT_DLU.f90 dlu_yeqax (y = A x) and dlu_yeqmaxpz (y = z - A x), face order
void KdifSolver::dlu_yeqax(const double* x, double* y) const {
  for (int c = 0; c < m->ncell; ++c) y[c] = dlu_diag[c] * x[c];
  for (int f = 0; f < m->nface; ++f) {
    const int lo = m->fc1[f], hi = m->fc2[f];
    y[hi] = y[hi] + dlu_lower[f] * x[lo];
    y[lo] = y[lo] + dlu_upper[f] * x[hi];
  }
}
void KdifSolver::dlu_yeqmaxpz(const double* x, const double* z, double* y) const {
  for (int c = 0; c < m->ncell; ++c) y[c] = z[c] - dlu_diag[c] * x[c];
  for (int f = 0; f < m->nface; ++f) {
    const int lo = m->fc1[f], hi = m->fc2[f];
    y[hi] = y[hi] - dlu_lower[f] * x[lo];
    y[lo] = y[lo] - dlu_upper[f] * x[hi];
  }
}

// dlu_cgs.f90:41-98: conjugate gradient squared, initial guess b / diag, stopped when the
// step |alpha| sum|u + q| falls below maxres sum|x0| or after max_it + 1 iterations; returns
// the iterations - 1, or -1 when not converged
int KdifSolver::dlu_cgs(std::vector<double>& sol, double maxres, int max_it) const {
  const int n = m->ncell;
  std::vector<double> r1(n), r2(n), p1(n), q1(n), u(n), v(n);
  auto dotp = [&](const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = s + a[i] * b[i];
    return s;
  };
  auto asum = [&](const std::vector<double>& a) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = s + std::fabs(a[i]);
    return s;
  };
  p1 = sol;
  for (int i = 0; i < n; ++i) sol[i] = p1[i] / dlu_diag[i];
  const double ref = asum(sol);
  dlu_yeqmaxpz(sol.data(), p1.data(), r1.data());
  r2 = r1;
  double err = std::numeric_limits<double>::max(), rho0 = 0.0;
  int nit = 0;
  while (err >= ref * maxres && nit <= max_it) {
    const double rho1 = dotp(r1, r2);
    if (nit == 0) {
      u = r1;
      p1 = r1;
    } else {
      const double beta = rho1 / rho0;
      for (int i = 0; i < n; ++i) u[i] = r1[i] + beta * q1[i];
      for (int i = 0; i < n; ++i) v[i] = q1[i] + beta * p1[i];
      for (int i = 0; i < n; ++i) p1[i] = u[i] + beta * v[i];
    }
    dlu_yeqax(p1.data(), v.data());
    const double alpha = rho1 / dotp(r2, v);
    for (int i = 0; i < n; ++i) q1[i] = u[i] - alpha * v[i];
    for (int i = 0; i < n; ++i) v[i] = u[i] + q1[i];
    err = std::fabs(alpha) * asum(v);
    for (int i = 0; i < n; ++i) sol[i] = sol[i] + alpha * v[i];
    dlu_yeqax(v.data(), u.data());
    for (int i = 0; i < n; ++i) r1[i] = r1[i] - alpha * u[i];
    rho0 = rho1;
    ++nit;
  }
  return nit <= max_it ? nit - 1 : -1;
}

// SPMAT_DLU.f90 dlu_yeqatx: y = A^T x
void KdifSolver::dlu_yeqatx(const double* x, double* y) const {
  for (int c = 0; c < m->ncell; ++c) y[c] = dlu_diag[c] * x[c];
  for (int f = 0; f < m->nface; ++f) {
    const int lo = m->fc1[f], hi = m->fc2[f];
    y[hi] = y[hi] + dlu_upper[f] * x[lo];
    y[lo] = y[lo] + dlu_lower[f] * x[hi];
  }
}

// dlu_bicg.f90: bi-conjugate gradients, stopped like dlu_cgs
int KdifSolver::dlu_bicg(std::vector<double>& sol, double maxres, int max_it) const {
  const int n = m->ncell;
  std::vector<double> r1(n), r2(n), p1(n), p2(n), q1(n), q2(n);
  auto dotp = [&](const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = s + a[i] * b[i];
    return s;
  };
  p1 = sol;
  for (int i = 0; i < n; ++i) sol[i] = p1[i] / dlu_diag[i];
  double ref = 0.0;
  for (int i = 0; i < n; ++i) ref = ref + std::fabs(sol[i]);
  dlu_yeqmaxpz(sol.data(), p1.data(), r1.data());
  r2 = r1;
  double err = std::numeric_limits<double>::max(), rho0 = 0.0;
  int nit = 0;
  while (err >= ref * maxres && nit <= max_it) {
    const double rho1 = dotp(r1, r2);
    if (nit == 0) {
      p1 = r1;
      p2 = r2;
    } else {
      const double beta = rho1 / rho0;
      for (int i = 0; i < n; ++i) p1[i] = r1[i] + beta * p1[i];
      for (int i = 0; i < n; ++i) p2[i] = r2[i] + beta * p2[i];
    }
    dlu_yeqax(p1.data(), q1.data());
    dlu_yeqatx(p2.data(), q2.data());
    const double alpha = rho1 / dotp(p2, q1);
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = s + std::fabs(p1[i]);
    err = std::fabs(alpha) * s;
    for (int i = 0; i < n; ++i) sol[i] = sol[i] + alpha * p1[i];
    for (int i = 0; i < n; ++i) r1[i] = r1[i] - alpha * q1[i];
    for (int i = 0; i < n; ++i) r2[i] = r2[i] - alpha * q2[i];
    rho0 = rho1;
    ++nit;
  }
  return nit <= max_it ? nit - 1 : -1;
}

// dlu_gmres.f90: restarted GMRES(nkrylov), modified Gram-Schmidt, Givens rotations
int KdifSolver::dlu_gmres(std::vector<double>& sol, double maxres, int max_it, int nk) const {
  const int n = m->ncell;
  auto dotp = [&](const double* a, const double* b) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = s + a[i] * b[i];
    return s;
  };
  std::vector<double> qc(nk + 1), qs(nk + 1), ss(nk + 2), yy(nk + 1), hh((size_t)(nk + 2) * (nk + 1));
  auto H = [&](int i, int j) -> double& { return hh[(size_t)i * (nk + 1) + j]; };  // 1-based
  std::vector<double> r1(n), p1(n), w1((size_t)nk * n), v1((size_t)nk * n);
  auto W = [&](int j) { return &w1[(size_t)(j - 1) * n]; };
  auto V = [&](int j) { return &v1[(size_t)(j - 1) * n]; };
  p1 = sol;
  for (int i = 0; i < n; ++i) sol[i] = p1[i] / dlu_diag[i];
  double ref = 0.0;
  for (int i = 0; i < n; ++i) ref = ref + std::fabs(sol[i]);
  const double normp1 = std::sqrt(dotp(p1.data(), p1.data()));
  const double eps = std::numeric_limits<double>::epsilon();
  double errgmres = std::numeric_limits<double>::max();
  int nit = 0;
  while (errgmres >= ref * maxres && nit <= max_it * 2) {
    dlu_yeqmaxpz(sol.data(), p1.data(), r1.data());
    const double beta = std::sqrt(dotp(r1.data(), r1.data()));
    double fact = 1.0 / beta;
    for (int i = 0; i < n; ++i) V(1)[i] = fact * r1[i];
    std::fill(ss.begin(), ss.end(), 0.0);
    ss[1] = beta;
    std::fill(hh.begin(), hh.end(), 0.0);
    int jk;
    for (jk = 1; jk <= nk; ++jk) {
      dlu_yeqax(V(jk), W(jk));
      for (int ik = 1; ik <= jk; ++ik) {
        H(ik, jk) = dotp(W(jk), V(ik));
        for (int i = 0; i < n; ++i) W(jk)[i] = W(jk)[i] - H(ik, jk) * V(ik)[i];
      }
      H(jk + 1, jk) = std::sqrt(dotp(W(jk), W(jk)));
      for (int ik = 1; ik <= jk - 1; ++ik) {
        const double tmp = H(ik, jk);
        H(ik, jk) = qc[ik] * tmp + qs[ik] * H(ik + 1, jk);
        H(ik + 1, jk) = -qs[ik] * tmp + qc[ik] * H(ik + 1, jk);
      }
      if (H(jk + 1, jk) > eps * 10 * normp1) {
        if (jk < nk) {
          fact = 1.0 / H(jk + 1, jk);
          for (int i = 0; i < n; ++i) V(jk + 1)[i] = fact * W(jk)[i];
        }
        if (H(jk, jk) == 0) break;
        const double tmp = std::sqrt(H(jk, jk) * H(jk, jk) + H(jk + 1, jk) * H(jk + 1, jk));
        qc[jk] = H(jk, jk) / tmp;
        qs[jk] = H(jk + 1, jk) / tmp;
        H(jk, jk) = tmp;
        H(jk + 1, jk) = 0.0;
        ss[jk + 1] = -qs[jk] * ss[jk];
        ss[jk] = qc[jk] * ss[jk];
        if (std::fabs(ss[jk + 1]) < maxres * std::fabs(ss[1])) break;
      } else {
        break;
      }
    }
    const int nkk = std::min(jk, nk);
    for (jk = nkk; jk >= 1; --jk) {
      double tmp = ss[jk];
      for (int ik = jk + 1; ik <= nkk; ++ik) tmp = tmp - H(jk, ik) * yy[ik];
      yy[jk] = tmp / H(jk, jk);
      for (int i = 0; i < n; ++i) sol[i] = sol[i] + yy[jk] * V(jk)[i];
    }
    dlu_yeqmaxpz(sol.data(), p1.data(), r1.data());
    ss[nkk + 1] = std::sqrt(dotp(r1.data(), r1.data()));
    errgmres = ss[nkk + 1] / normp1;
    ++nit;
  }
  return nit <= max_it ? nit - 1 : -1;
}

void kdif_typhon_steady(KdifSolver& k, std::vector<double>& U, const KdifSteadyParams& p, KdifSteadyOut& out) {
  const UMesh* m = k.m;
  const int nc = m->ncell, nci = m->ncell_int;
  // calc_refcons.f90: volume average of U; zone_preproc.f90: total volume
  double refsca = 0.0, totvol = 0.0;
  for (int c = 0; c < nci; ++c) refsca = refsca + U[c] * m->cvol[c];
  for (int c = 0; c < nci; ++c) totvol = totvol + m->cvol[c];
  refsca = refsca / totvol;
  const double tiny = std::numeric_limits<double>::min();
  double w_ref = 1.0, w_cur = 1.0, z_reforig = 0.0;
  int iter_tot = 0;
  std::vector<double> x(nc);
  for (int icycle = 1; icycle <= p.max_cycles; ++icycle) {
    w_cur = tiny;
    double z_ref = w_cur, z_cur = z_ref;
    const int maxit = p.max_iters - iter_tot;
    int iter_loc = 0;
    bool end = false;
    while (!end) {
      ++iter_loc;
      ++iter_tot;
      const double dt = k.fourier_dt(p.fourier, p.conduct);
      for (int c = 0; c < nci; ++c) k.T[c] = U[c] / k.cp;  // calc_varprim_kdif
      k.rhs(dt);
      k.typhon_dlu(dt);
      for (int c = 0; c < nc; ++c) x[c] = c < nci ? k.residu[c] : 0.0;
      if (p.inversion == 1) k.dlu_bicg(x, p.cgs_maxres, p.cgs_max_it);
      else if (p.inversion == 2) k.dlu_gmres(x, p.cgs_maxres, p.cgs_max_it, p.nkrylov);
      else k.dlu_cgs(x, p.cgs_maxres, p.cgs_max_it);
      double s = 0.0;  // update_field.f90: U += dU, residual sum|dU| / refsca
      for (int c = 0; c < nci; ++c) {
        U[c] = U[c] + x[c];
        s = s + std::fabs(x[c]);
      }
      z_cur = 0.0 + s / refsca;
      z_ref = std::max(z_ref, z_cur);  // check_end_cycle.f90
      if (z_cur / z_ref <= p.cycle_res) end = true;
      if (iter_loc == maxit) end = true;
      out.log_res.push_back(std::log10(z_cur));
    }
    if (icycle == 1) z_reforig = z_ref;
    if (z_cur / z_reforig >= w_cur / w_ref) {
      w_cur = z_cur;
      w_ref = z_reforig;
    }
    double tv = 0.0, vol = 0.0;  // VOL_AVERAGE probe of the temperature
    for (int c = 0; c < nci; ++c) tv = tv + (U[c] / k.cp) * m->cvol[c];
    for (int c = 0; c < nci; ++c) vol = vol + m->cvol[c];
    out.cycle_avg.push_back(tv / vol);
    out.cycle_end.push_back(iter_tot);
    if (w_cur / w_ref <= p.global_res || iter_tot >= p.max_iters) break;
  }
  for (int c = 0; c < nci; ++c) k.T[c] = U[c] / k.cp;
}

}  // namespace ory
