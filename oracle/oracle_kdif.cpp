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

}  // namespace ory
