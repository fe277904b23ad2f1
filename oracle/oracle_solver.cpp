// Typhon CPU oracle — explicit Euler path.  TEST INFRASTRUCTURE ONLY (see oracle.hpp).
//
// Each routine restates one Typhon routine in its loop and summation order:
//   varprim          SOURCE/EQNS/calc_varprim_ns.f90:37-57
//   varcons          SOURCE/EQNS/calc_varcons_ns.f90:30-48
//   boco_*           SOURCE/MGRID/calcboco_gen.f90:40-88, calcboco_connect_per_match.f90:45-84,
//                    SOURCE/MGRID/calcboco_ust_sym.f90 (symmetry), calcboco_ust.f90
//   precalc_grad_lsq SOURCE/MGRID/precalc_grad_lsq.f90:43-159, SOURCE/MATH/MATRIX.f90:42-70
//   calc_gradient    SOURCE/MGRID/calc_gradient.f90:67-196, MATRIX.f90:79-111
//   hres_states      SOURCE/MAIN/calc_hres_states.f90:55-119, SOURCE/EQNS/hres_ns_muscl*.f90,
//                    SOURCE/EQNS/tvdgrad{str,fst,uns}_{scal,vect}.f90, SOURCE/MGRID/LIMITER.f90
//   postlimit_barth  SOURCE/MGRID/postlimit_barth.f90:42-223
//   face_fluxes      SOURCE/EQNS/calc_flux_hllc.f90:61-171, calc_roe_states.f90:35-53,
//                    calc_flux_rusanov.f90:57-83; Roe: new (no Typhon implementation)
//   flux_to_res      SOURCE/MAIN/flux_to_res.f90:47-144
//   timestep         SOURCE/EQNS/calc_ns_timestep.f90:52-103, SOURCE/ZONE/calc_zonetimestep.f90:54-126
//   rk_step          SOURCE/MAIN/treelevel_rungekutta.f90:48-113, SOURCE/ZONE/update_field.f90:33-71,
//                    SOURCE/PARAM/MENU_NUM.f90:368-449
#include <algorithm>
#include <cmath>
#include <limits>

#include "oracle.hpp"

namespace ory {

RkTable rk_table(int method) {
  RkTable t;
  auto set = [&](int n, std::initializer_list<std::initializer_list<double>> rows) {
    t.nstage = n;
    t.coef.assign((size_t)n * n, 0.0);
    int i = 0;
    for (auto& r : rows) {
      int j = 0;
      for (double v : r) t.coef[(size_t)i * n + j++] = v;
      ++i;
    }
  };
  switch (method) {
    case EXPLICIT: set(1, {{1.}}); break;  // treelevel_explicit.f90: calc_rhs, then U += residu
    case RK2: set(2, {{.5}, {0., 1.}}); break;
    case RK2SSP: set(2, {{1.}, {.5, .5}}); break;
    case RK3SSP: set(3, {{1.}, {.25, .25}, {1. / 6., 1. / 6., 4. / 6.}}); break;
    case RK4: set(4, {{.5}, {0., .5}, {0., 0., 1.}, {1. / 6., 2. / 6., 2. / 6., 1. / 6.}}); break;
    case LSRK25BB:
      set(5, {{0.1815754863270908}, {0., 0.238260222208392}, {0., 0., 0.330500707328},
              {0., 0., 0., 0.5}, {0., 0., 0., 0., 1.}});
      break;
    case LSRK26BB:
      set(6, {{0.11797990162882}, {0., 0.18464696649448}, {0., 0., 0.24662360430959},
              {0., 0., 0., 0.33183954253762}, {0., 0., 0., 0., 0.5}, {0., 0., 0., 0., 0., 1.}});
      break;
    case LSRK12BS: set(2, {{1.}, {0., 1.}}); break;
    case LSRK13BS: set(3, {{.15}, {0., .4}, {0., 0., 1.}}); break;
    default: break;
  }
  return t;
}

void Solver::init(const UMesh* mesh, const SpatParams& p, int rk_method, double cfl_) {
  m = mesh;
  sp = p;
  rk = rk_table(rk_method);
  cfl = cfl_;
  const size_t nc = m->ncell, nf = m->nface;
  cons.assign(5 * nc, 0.0);
  prim.assign(5 * nc, 0.0);
  grad.assign(15 * nc, 0.0);
  cell_l.assign(5 * nf, 0.0);
  cell_r.assign(5 * nf, 0.0);
  flux.assign(5 * nf, 0.0);
  residu.assign(5 * nc, 0.0);
  dtloc.assign(nc, 0.0);
  limratio.assign(3 * nc, 1.0);
  gradcond_ok = false;
}

// calc_varprim_ns.f90:43-54, over all cells (ghosts too)
void Solver::varprim() {
  const int nc = m->ncell;
  const double g1 = sp.gamma - 1.0;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nc; ++i) {
    double rho = cons[i];
    V3 vel = v3(cons[2 * nc + i], cons[3 * nc + i], cons[4 * nc + i]) / rho;
    double ec = 0.5 * rho * sqrabs(vel);
    prim[i] = rho;
    prim[nc + i] = g1 * (cons[nc + i] - ec);
    prim[2 * nc + i] = vel.x;
    prim[3 * nc + i] = vel.y;
    prim[4 * nc + i] = vel.z;
  }
}

// calc_varcons_ns.f90:37-46
void Solver::varcons() {
  const int nc = m->ncell;
  const double ig1 = 1.0 / (sp.gamma - 1.0);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nc; ++i) {
    double rho = prim[i];
    V3 vel = v3(prim[2 * nc + i], prim[3 * nc + i], prim[4 * nc + i]);
    cons[i] = rho;
    cons[nc + i] = ig1 * prim[nc + i] + 0.5 * rho * sqrabs(vel);
    cons[2 * nc + i] = rho * vel.x;
    cons[3 * nc + i] = rho * vel.y;
    cons[4 * nc + i] = rho * vel.z;
  }
}

// calcboco_gen(bccon_cell_state): periodic copy (calcboco_connect_per_match.f90:56-78) and
// physical ghost states (calcboco_ust.f90 -> calcboco_ust_sym / wall)
// d(ghost conservative state)/d(inside conservative state) of the far-field kinds, row-major
// in (rho, rhoE, rhou, rhov, rhow); u is the inside velocity.  Returns false for the
// supersonic inflow (ghost independent of the inside state).
bool farfield_jacobian(double gamma, const double* qinf, V3 n, const double* q, double* M) {
  const double vn = qinf[2] * n.x + qinf[3] * n.y + qinf[4] * n.z;
  const double c = std::sqrt(gamma * qinf[1] / qinf[0]);
  for (int k = 0; k < 25; ++k) M[k] = 0.0;
  if (vn <= -c) return false;
  const double u2 = q[2] * q[2] + q[3] * q[3] + q[4] * q[4];
  if (vn < -1e-8 * c) {      // subsonic inflow: rhoE_g = p / (gamma - 1) + const
    M[5] = 0.5 * u2; M[6] = 1.0; M[7] = -q[2]; M[8] = -q[3]; M[9] = -q[4];
  } else if (vn < c) {       // subsonic outflow: rho, rhou kept, rhoE_g = p_inf / (gamma - 1) + |m|^2 / (2 rho)
    M[0] = 1.0;
    M[5] = -0.5 * u2; M[7] = q[2]; M[8] = q[3]; M[9] = q[4];
    M[12] = 1.0; M[18] = 1.0; M[24] = 1.0;
  } else {                   // supersonic outflow: identity
    for (int i = 0; i < 5; ++i) M[i * 6] = 1.0;
  }
  return true;
}

// d(ghost conservative state)/d(inside conservative state) of the no-slip wall face state
// (rho_g = rho, p_g = p, u_g = 2 u_w - u): rho E_g = rho E + 2 rho |u_w|^2 - 2 u_w.m,
// m_g = 2 rho u_w - m (new; Typhon folds no wall Jacobian)
void noslip_jacobian(V3 uw, double* M) {
  const double w[3] = {uw.x, uw.y, uw.z};
  for (int k = 0; k < 25; ++k) M[k] = 0.0;
  M[0] = 1.0;
  M[5] = 2.0 * (w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  M[6] = 1.0;
  for (int j = 0; j < 3; ++j) M[7 + j] = -2.0 * w[j];
  for (int i = 0; i < 3; ++i) {
    M[(2 + i) * 5] = 2.0 * w[i];
    M[(2 + i) * 5 + 2 + i] = -1.0;
  }
}

void farfield_state(double gamma, const double* qinf, V3 n, const double* q, double* out) {
  const double vn = qinf[2] * n.x + qinf[3] * n.y + qinf[4] * n.z;
  const double c = std::sqrt(gamma * qinf[1] / qinf[0]);
  if (vn <= -c) {
    for (int v = 0; v < 5; ++v) out[v] = qinf[v];
  } else if (vn < -1e-8 * c) {
    out[0] = qinf[0]; out[1] = q[1]; out[2] = qinf[2]; out[3] = qinf[3]; out[4] = qinf[4];
  } else if (vn < c) {
    out[0] = q[0]; out[1] = qinf[1]; out[2] = q[2]; out[3] = q[3]; out[4] = q[4];
  } else {
    for (int v = 0; v < 5; ++v) out[v] = q[v];
  }
}

// Isentropic conversions of EQNS.f90:139-219 on one primitive state q = (rho, p, u, v, w)
static V3 unit_dir(const double* d) {  // dir / abs(dir)
  V3 v = v3(d[0], d[1], d[2]);
  const double a = std::sqrt(sqrabs(v));
  return v3(v.x / a, v.y / a, v.z / a);
}
static void pi_ti_mach_dir2prim(double g, double r, double pi, double ti, double mach, V3 dir, double* q) {
  const double g1 = g - 1.0;
  const double fm = 1.0 / (1.0 + .5 * g1 * (mach * mach));
  const double ts = ti * fm;
  const double a = std::sqrt(g * r * ts);
  q[1] = pi * std::pow(fm, g / g1);
  q[0] = q[1] / (r * ts);
  const V3 u = (mach * a) * dir;
  q[2] = u.x; q[3] = u.y; q[4] = u.z;
}
static void pi_ti_ps_dir2prim(double g, double r, double pi, double ti, double ps, V3 dir, double* q) {
  const double g1 = g - 1.0;
  double fm = std::pow(pi / ps, g1 / g);
  if (fm < 1.0) fm = 1.0;  // "Bad ratio Pi/P : truncated to 1."
  q[1] = ps;
  q[0] = ps / (r * ti) * fm;
  const V3 u = (std::sqrt((fm - 1.0) * 2.0 / g1) * std::sqrt(g * ps / q[0])) * dir;
  q[2] = u.x; q[3] = u.y; q[4] = u.z;
}
static void prim2pi_ti_mach_dir(double g, double r, const double* q, double& pi, double& ti, double& mach, V3& dir) {
  const double g1 = g - 1.0;
  const V3 u = v3(q[2], q[3], q[4]);
  double fmv = sqrabs(u);
  const double n = std::sqrt(fmv);
  dir = v3(u.x / n, u.y / n, u.z / n);
  fmv = fmv / (g * q[1]) * q[0];
  mach = std::sqrt(fmv);
  fmv = 1.0 + 0.5 * g1 * fmv;
  pi = q[1] * std::pow(fmv, g / g1);
  ti = q[1] / r / q[0] * fmv;
}

// Inlet / outlet state from the inside state qi (setboco_ns_inlet_sub.f90:64-96,
// setboco_ns_outlet_sub.f90:31-60, setboco_ns_inlet_sup.f90:75-101, setboco_ns_outlet_sup.f90)
void inout_state(int kind, double g, double r, const double* data, const double* qi, double* qo) {
  if (kind == BC_INLET_SUB) {
    pi_ti_ps_dir2prim(g, r, data[0], data[1], qi[1], unit_dir(data + 2), qo);
  } else if (kind == BC_OUTLET_SUB) {
    double pi, ti, mach;
    V3 dir;
    prim2pi_ti_mach_dir(g, r, qi, pi, ti, mach, dir);
    pi_ti_ps_dir2prim(g, r, pi, ti, data[0], dir, qo);
  } else if (kind == BC_INLET_SUP) {
    pi_ti_mach_dir2prim(g, r, data[0], data[1], data[2], unit_dir(data + 3), qo);
  } else {
    for (int v = 0; v < 5; ++v) qo[v] = qi[v];
  }
}

void Solver::boco_cell_state() {
  const int nc = m->ncell;
  for (auto& b : m->bocos) {
    for (size_t k = 0; k < b.iface.size(); ++k) {
      int f = b.iface[k];
      int g = m->fc2[f];
      if (b.kind == BC_PERIODIC) {
        int s = m->fc1[b.partner_face[k]];
        for (int v = 0; v < 5; ++v) prim[v * nc + g] = prim[v * nc + s];
        if (b.rotation) {  // transvec_per: the velocity rotated into this family's frame
          V3 u = rot_apply(b.rot, v3(prim[2 * nc + s], prim[3 * nc + s], prim[4 * nc + s]));
          prim[2 * nc + g] = u.x; prim[3 * nc + g] = u.y; prim[4 * nc + g] = u.z;
        }
      } else if (b.kind == BC_SYMMETRY) {
        // calcboco_ust_sym: mirror the velocity across the face plane
        int i = m->fc1[f];
        V3 fn = m->fnormal[f];
        V3 u = v3(prim[2 * nc + i], prim[3 * nc + i], prim[4 * nc + i]);
        V3 ug = u - (2.0 * dot(u - V3(), fn)) * fn;
        prim[g] = prim[i];
        prim[nc + g] = prim[nc + i];
        prim[2 * nc + g] = ug.x;
        prim[3 * nc + g] = ug.y;
        prim[4 * nc + g] = ug.z;
      } else if (b.kind == BC_WALL || b.kind == BC_NOSLIP) {
        // setboco_ns_flux.f90, cell-state mode, adiabatic wall (lflux = 0): ghost pressure
        // = cell pressure, ghost temperature = cell temperature - lflux d / conduct, velocity
        // reflected about the wall velocity
        int i = m->fc1[f];
        const double r = sp.rgas;
        const double lflux = 0.0;
        V3 cgface = m->fcentre[f], cg = m->ccentre[i], nrm = m->fnormal[f];
        double d = dot(cgface - cg, cgface - cg) / std::fabs(dot(cgface - cg, nrm));
        double mu = viscosity(prim[i], prim[nc + i] / (r * prim[i]));
        double cp = sp.gamma / (sp.gamma - 1.0) * r;
        double conduct = mu * cp / sp.prandtl;
        double temp = prim[nc + i] / (prim[i] * r) - lflux * d / conduct;
        prim[nc + g] = prim[nc + i];
        prim[g] = prim[nc + g] / (r * temp);
        V3 u = v3(prim[2 * nc + i], prim[3 * nc + i], prim[4 * nc + i]);
        V3 ug = (2.0 * b.wall_velocity) - u;
        prim[2 * nc + g] = ug.x;
        prim[3 * nc + g] = ug.y;
        prim[4 * nc + g] = ug.z;
      } else if (b.kind == BC_FARFIELD) {
        int i = m->fc1[f];
        double q[5], o[5];
        for (int v = 0; v < 5; ++v) q[v] = prim[v * nc + i];
        farfield_state(sp.gamma, sp.farfield, m->fnormal[f], q, o);
        for (int v = 0; v < 5; ++v) prim[v * nc + g] = o[v];
      } else if (b.kind >= BC_INLET_SUB && b.kind <= BC_OUTLET_SUP) {
        int i = m->fc1[f];
        double q[5], o[5];
        for (int v = 0; v < 5; ++v) q[v] = prim[v * nc + i];
        inout_state(b.kind, sp.gamma, sp.rgas, b.data, q, o);
        for (int v = 0; v < 5; ++v) prim[v * nc + g] = o[v];
      }
    }
  }
}

// calcboco_gen(bccon_cell_grad): connections only (calcboco_gen.f90:78-84)
void Solver::boco_cell_grad() {
  const int nc = m->ncell;
  for (auto& b : m->bocos) {
    if (b.kind != BC_PERIODIC) continue;
    for (size_t k = 0; k < b.iface.size(); ++k) {
      int g = m->fc2[b.iface[k]];
      int s = m->fc1[b.partner_face[k]];
      for (int v = 0; v < 15; ++v) grad[v * nc + g] = grad[v * nc + s];
      if (b.rotation) {
        // scalar gradients: vectors, R g (transvec_per); the velocity gradient tensor
        // G(i,j) = du_i/dx_j: G R^T (transten_per -> t3d_rot, TENSOR3.f90:328-340)
        const double* R = b.rot;
        for (int q = 0; q < 2; ++q) {
          V3 gq = rot_apply(R, v3(grad[(3 * q) * nc + s], grad[(3 * q + 1) * nc + s], grad[(3 * q + 2) * nc + s]));
          grad[(3 * q) * nc + g] = gq.x; grad[(3 * q + 1) * nc + g] = gq.y; grad[(3 * q + 2) * nc + g] = gq.z;
        }
        for (int i = 0; i < 3; ++i) {
          double G[3];
          for (int j = 0; j < 3; ++j) G[j] = grad[(6 + 3 * i + j) * nc + s];
          for (int j = 0; j < 3; ++j) grad[(6 + 3 * i + j) * nc + g] = G[0] * R[3 * j] + G[1] * R[3 * j + 1] + G[2] * R[3 * j + 2];
        }
      }
    }
  }
}

// calcboco_gen(bccon_face_state): periodic cell_r(face) = cell_l(partner face)
// (calcboco_connect_per_match.f90:56-78); symmetry cell_r(face) = cell_l(face) with the
// velocity mirrored across the face (calcboco_ust_sym.f90, face-state mode)
void Solver::boco_face_state() {
  const int nf = m->nface;
  for (auto& b : m->bocos) {
    for (size_t k = 0; k < b.iface.size(); ++k) {
      int f = b.iface[k];
      if (b.kind == BC_PERIODIC) {
        int fp = b.partner_face[k];
        for (int v = 0; v < 5; ++v) cell_r[v * nf + f] = cell_l[v * nf + fp];
        if (b.rotation) {
          V3 u = rot_apply(b.rot, v3(cell_l[2 * nf + fp], cell_l[3 * nf + fp], cell_l[4 * nf + fp]));
          cell_r[2 * nf + f] = u.x; cell_r[3 * nf + f] = u.y; cell_r[4 * nf + f] = u.z;
        }
      } else if (b.kind == BC_WALL || b.kind == BC_NOSLIP) {
        // setboco_ns_flux.f90, face-state mode: cell_r takes cell_l's PRESSURE as its density
        // ("weak BC"), cell_l's pressure, and the velocity reflected about the wall velocity;
        // BC_NOSLIP (new) takes cell_l's density
        cell_r[f] = b.kind == BC_NOSLIP ? cell_l[f] : cell_l[nf + f];
        cell_r[nf + f] = cell_l[nf + f];
        V3 u = v3(cell_l[2 * nf + f], cell_l[3 * nf + f], cell_l[4 * nf + f]);
        V3 ug = (2.0 * b.wall_velocity) - u;
        cell_r[2 * nf + f] = ug.x;
        cell_r[3 * nf + f] = ug.y;
        cell_r[4 * nf + f] = ug.z;
      } else if (b.kind == BC_SYMMETRY) {
        V3 fn = m->fnormal[f];
        V3 u = v3(cell_l[2 * nf + f], cell_l[3 * nf + f], cell_l[4 * nf + f]);
        V3 ug = u - (2.0 * dot(u - V3(), fn)) * fn;
        cell_r[f] = cell_l[f];
        cell_r[nf + f] = cell_l[nf + f];
        cell_r[2 * nf + f] = ug.x;
        cell_r[3 * nf + f] = ug.y;
        cell_r[4 * nf + f] = ug.z;
      } else if (b.kind == BC_FARFIELD) {
        double q[5], o[5];
        for (int v = 0; v < 5; ++v) q[v] = cell_l[v * nf + f];
        farfield_state(sp.gamma, sp.farfield, m->fnormal[f], q, o);
        for (int v = 0; v < 5; ++v) cell_r[v * nf + f] = o[v];
      } else if (b.kind >= BC_INLET_SUB && b.kind <= BC_OUTLET_SUP) {
        double q[5], o[5];
        for (int v = 0; v < 5; ++v) q[v] = cell_l[v * nf + f];
        inout_state(b.kind, sp.gamma, sp.rgas, b.data, q, o);
        for (int v = 0; v < 5; ++v) cell_r[v * nf + f] = o[v];
      }
    }
  }
}

// MATRIX.f90:42-70 (cholesky_decomp), a column-major 3x3: a(i,j) = a[(j-1)*3 + (i-1)]
static void cholesky_decomp(double* a) {
  auto A = [&](int i, int j) -> double& { return a[(j - 1) * 3 + (i - 1)]; };
  for (int i = 1; i <= 3; ++i)
    for (int j = i; j <= 3; ++j) {
      double sum = A(i, j);
      for (int k = i - 1; k >= 1; --k) sum = sum - A(i, k) * A(j, k);
      if (i == j) A(i, i) = std::sqrt(sum);
      else A(j, i) = sum / A(i, i);
    }
}
// MATRIX.f90:79-111 (cholesky_solve), b(3, p) column-major
static void cholesky_solve(const double* a, double* b, int p) {
  auto A = [&](int i, int j) { return a[(j - 1) * 3 + (i - 1)]; };
  auto B = [&](int i, int k) -> double& { return b[(k - 1) * 3 + (i - 1)]; };
  for (int i = 1; i <= 3; ++i) {
    for (int j = 1; j <= i - 1; ++j)
      for (int k = 1; k <= p; ++k) B(i, k) = B(i, k) - A(i, j) * B(j, k);
    for (int k = 1; k <= p; ++k) B(i, k) = B(i, k) / A(i, i);
  }
  for (int i = 3; i >= 1; --i) {
    for (int j = i + 1; j <= 3; ++j)
      for (int k = 1; k <= p; ++k) B(i, k) = B(i, k) - A(j, i) * B(j, k);
    for (int k = 1; k <= p; ++k) B(i, k) = B(i, k) / A(i, i);
  }
}

// precalc_grad_lsq.f90:43-159
void Solver::precalc_grad_lsq() {
  const int nci = m->ncell_int, nf = m->nface, nfi = m->nface_int;
  gradcond.assign(9 * (size_t)nci, 0.0);
  std::vector<V3> dcg(nf);
  for (int f = 0; f < nf; ++f) {
    dcg[f] = m->ccentre[m->fc2[f]] - m->ccentre[m->fc1[f]];
    if (sp.gradmeth == GRAD_LSQW) dcg[f] = dcg[f] / sqrabs(dcg[f]);
  }
  auto add = [&](int c, const V3& d) {
    double im[9];
    im[0] = d.x * d.x; im[4] = d.y * d.y; im[8] = d.z * d.z;
    im[3] = d.x * d.y; im[1] = im[3];
    im[6] = d.x * d.z; im[2] = im[6];
    im[7] = d.y * d.z; im[5] = im[7];
    for (int k = 0; k < 9; ++k) gradcond[9 * (size_t)c + k] = gradcond[9 * (size_t)c + k] + im[k];
  };
  for (int f = 0; f < nfi; ++f) { add(m->fc1[f], dcg[f]); add(m->fc2[f], dcg[f]); }
  for (int f = nfi; f < nf; ++f) add(m->fc1[f], dcg[f]);
  if (m->dim == 2)
    for (int c = 0; c < nci; ++c) gradcond[9 * (size_t)c + 8] = gradcond[9 * (size_t)c + 8] + 1.0;
  for (int c = 0; c < nci; ++c) cholesky_decomp(&gradcond[9 * (size_t)c]);
  gradcond_ok = true;
}

// calc_gradient.f90:67-196 (5 components: rho, p, u, v, w)
void Solver::calc_gradient() {
  if (!gradcond_ok) precalc_grad_lsq();
  const int nc = m->ncell, nci = m->ncell_int, nf = m->nface, nfi = m->nface_int;
  std::vector<V3> dcg(nf);
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    V3 d = m->ccentre[m->fc2[f]] - m->ccentre[m->fc1[f]];
    if (sp.gradmeth == GRAD_LSQW) {
      double s = sqrabs(d);
      d = d / (s * s);
    }
    dcg[f] = d;
  }
  // rhs(1:3, ic*dim + dec), dim = 5: per cell a column-major 3x5 block
  std::vector<double> rhs(15 * (size_t)nci, 0.0);
  for (auto& col : m->colors)  // faces of one colour touch distinct cells
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < col.size(); ++q) {
      const int f = col[q];
      int i1 = m->fc1[f], i2 = m->fc2[f];
      for (int v = 0; v < 5; ++v) {
        double dsca = prim[v * nc + i2] - prim[v * nc + i1];
        double* r1 = &rhs[15 * (size_t)i1 + 3 * v];
        r1[0] = r1[0] + dsca * dcg[f].x;
        r1[1] = r1[1] + dsca * dcg[f].y;
        r1[2] = r1[2] + dsca * dcg[f].z;
        if (f < nfi) {
          double* r2 = &rhs[15 * (size_t)i2 + 3 * v];
          r2[0] = r2[0] + dsca * dcg[f].x;
          r2[1] = r2[1] + dsca * dcg[f].y;
          r2[2] = r2[2] + dsca * dcg[f].z;
        }
      }
    }
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nci; ++c) cholesky_solve(&gradcond[9 * (size_t)c], &rhs[15 * (size_t)c], 5);
  // grad%tabvect(is) for rho, p; grad%tabtens(1)%mat(i, 1:3) = rhs(1:3, nscal + i)
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nci; ++c)
    for (int v = 0; v < 5; ++v)
      for (int k = 0; k < 3; ++k) grad[(3 * v + k) * (size_t)nc + c] = rhs[15 * (size_t)c + 3 * v + k];
}

// ---------------------------------------------------------------------------
// Limiters (LIMITER.f90).  Scalars go through the array forms (*_t), vector components
// through the scalar forms (called by *_vt), as in tvdgrad*_{scal,vect}.
static double sgn1(double x) { return std::signbit(x) ? -1.0 : 1.0; }
static double lim_scalar_form(int lim, double x1, double x2) {
  switch (lim) {
    case LIM_MINMOD: {  // LIMITER.f90:72-82
      double s = 0.5 * (sgn1(x1) + sgn1(x2));
      return s * std::min(std::fabs(x1), std::fabs(x2));
    }
    case LIM_ALBADA: {  // LIMITER.f90:122-133
      double s = x1 * x2;
      if (s <= 0.0) return 0.0;
      return s * (x1 + x2) / (x1 * x1 + x2 * x2);
    }
    case LIM_VLEER: {
      double s = x1 * x2;
      if (s <= 0.0) return 0.0;
      return 2.0 * s / (x1 + x2);
    }
    case LIM_SBEE: {
      double r = 0.0;
      if (x1 > 0.0 && x2 > 0.0) r = std::max(std::min(2.0 * x1, x2), std::min(2.0 * x2, x1));
      if (x1 < 0.0 && x2 < 0.0) r = std::min(std::max(2.0 * x1, x2), std::max(2.0 * x2, x1));
      return r;
    }
    case LIM_KIM3: {
      double r = 0.0;
      if (x1 > 0.0 && x2 > 0.0) { r = (2.0 * x1 + x2) / 3.0; r = std::min(std::min(2.0 * x1, 2.0 * x2), r); }
      if (x1 < 0.0 && x2 < 0.0) { r = (2.0 * x1 + x2) / 3.0; r = std::max(std::max(2.0 * x1, 2.0 * x2), r); }
      return r;
    }
    case LIM_LIM03: {
      double eta = (x1 * x1 + x2 * x2) / 0.01 / 0.01;
      double r = 0.0;
      if (eta < 1.0) r = (2.0 * x2 + x1) / 3.0;
      else if (x1 > 0.0 && x2 > 0.0) { r = (2.0 * x2 + x1) / 3.0; r = std::min(std::min(1.6 * x2, 2.0 * x1), r); }
      else if (x1 < 0.0 && x2 < 0.0) { r = (2.0 * x2 + x1) / 3.0; r = std::max(std::max(1.6 * x2, 2.0 * x1), r); }
      else if (x1 < 0.0 && x2 > 0.0) { r = (2.0 * x2 + x1) / 3.0; r = std::max(0.0, std::min(-0.5 * x1, r)); }
      else if (x1 > 0.0 && x2 < 0.0) { r = (2.0 * x2 + x1) / 3.0; r = std::min(0.0, std::max(-0.5 * x1, r)); }
      return r;
    }
  }
  return 0.0;
}
static double lim_array_form(int lim, double x1, double x2) {
  switch (lim) {
    case LIM_MINMOD:  // LIMITER.f90:85-92
      if (x1 > 0.0 && x2 > 0.0) return std::min(x1, x2);
      if (x1 < 0.0 && x2 < 0.0) return std::max(x1, x2);
      return 0.0;
    case LIM_ALBADA:  // LIMITER.f90:136-144
      if ((x1 > 0.0 && x2 > 0.0) || (x1 < 0.0 && x2 < 0.0))
        return x1 * x2 * (x1 + x2) / (x1 * x1 + x2 * x2);
      return 0.0;
    case LIM_VLEER:
      if ((x1 > 0.0 && x2 > 0.0) || (x1 < 0.0 && x2 < 0.0)) return 2.0 * x1 * x2 / (x1 + x2);
      return 0.0;
    default:
      return lim_scalar_form(lim, x1, x2);
  }
}
// limiter applied to the MUSCL slopes: fast/str use lim(2g - LR, LR), uns uses lim(g, LR);
// kim3 swaps its arguments (tvdgrad*.f90)
static double apply_lim(int lim, bool uns, bool arrayform, double g, double LR) {
  double a = uns ? g : 2.0 * g - LR, b = LR;
  if (lim == LIM_KIM3) std::swap(a, b);
  return arrayform ? lim_array_form(lim, a, b) : lim_scalar_form(lim, a, b);
}

void Solver::hres_states() {
  const int nc = m->ncell, nf = m->nface;
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    const int icl = m->fc1[f], icr = m->fc2[f];
    if (sp.highres == HRES_NONE) {  // distrib_field.f90
      for (int v = 0; v < 5; ++v) {
        cell_l[v * nf + f] = prim[v * nc + icl];
        cell_r[v * nf + f] = prim[v * nc + icr];
      }
      continue;
    }
    const V3 CL = m->ccentre[icl], CR = m->ccentre[icr], F = m->fcentre[f];
    V3 uLR = CR - CL;
    double dLR;
    double kLF = 0, kRF = 0;
    V3 LF, RF;
    if (sp.highres == HRES_MUSCLFAST) {  // hres_ns_musclfast.f90:40-50
      kLF = vabs(F - CL);
      kRF = -vabs(F - CR);
      dLR = kLF - kRF;
      uLR = uLR / dLR;
    } else {  // hres_ns_muscl.f90 / hres_ns_muscluns.f90:40-50
      LF = F - CL;
      RF = F - CR;
      dLR = vabs(uLR);
      uLR = uLR / dLR;
    }
    const bool uns = sp.highres == HRES_MUSCLUNS;
    double dL[5], dR[5];
    // scalars (rho, p)
    for (int s = 0; s < 2; ++s) {
      double LRsca = (prim[s * nc + icr] - prim[s * nc + icl]) / dLR;
      for (int side = 0; side < 2; ++side) {
        int c = side == 0 ? icl : icr;
        V3 vg = v3(grad[(3 * s) * (size_t)nc + c], grad[(3 * s + 1) * (size_t)nc + c],
                   grad[(3 * s + 2) * (size_t)nc + c]);
        double out;
        if (sp.highres == HRES_MUSCLFAST) {  // tvdgradfst_scal.f90:35-57
          double sg;
          if (sp.limiter == LIM_NONE) sg = LRsca;
          else sg = apply_lim(sp.limiter, false, true, dot(vg, uLR), LRsca);
          out = sg * (side == 0 ? kLF : kRF);
        } else {  // tvdgradstr_scal.f90 / tvdgraduns_scal.f90:35-57
          double sg = dot(vg, uLR);
          if (sp.limiter == LIM_NONE) sg = LRsca - sg;
          else sg = apply_lim(sp.limiter, uns, true, sg, LRsca) - sg;
          vg = vg + sg * uLR;
          out = dot(vg, side == 0 ? LF : RF);
        }
        (side == 0 ? dL : dR)[s] = out;
      }
    }
    // velocity (tensor gradient)
    {
      V3 qL = v3(prim[2 * nc + icl], prim[3 * nc + icl], prim[4 * nc + icl]);
      V3 qR = v3(prim[2 * nc + icr], prim[3 * nc + icr], prim[4 * nc + icr]);
      V3 LRvec = (qR - qL) / dLR;
      for (int side = 0; side < 2; ++side) {
        int c = side == 0 ? icl : icr;
        double T[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) T[i][j] = grad[(6 + 3 * i + j) * (size_t)nc + c];
        auto matvec = [&](const V3& v) {
          // matmul(t%mat, tab(v)) (TENSOR3.f90:255-262)
          return v3(T[0][0] * v.x + T[0][1] * v.y + T[0][2] * v.z,
                    T[1][0] * v.x + T[1][1] * v.y + T[1][2] * v.z,
                    T[2][0] * v.x + T[2][1] * v.y + T[2][2] * v.z);
        };
        V3 vc = matvec(uLR);
        double lrv[3] = {LRvec.x, LRvec.y, LRvec.z};
        double vcc[3] = {vc.x, vc.y, vc.z};
        double out[3];
        if (sp.highres == HRES_MUSCLFAST) {  // tvdgradfst_vect.f90:35-58
          double k = side == 0 ? kLF : kRF;
          for (int i = 0; i < 3; ++i) {
            double s = sp.limiter == LIM_NONE ? lrv[i] : apply_lim(sp.limiter, false, false, vcc[i], lrv[i]);
            out[i] = k * s;
          }
        } else {  // tvdgradstr_vect.f90 / tvdgraduns_vect.f90:36-58
          double s[3];
          for (int i = 0; i < 3; ++i) {
            if (sp.limiter == LIM_NONE) s[i] = lrv[i] - vcc[i];
            else s[i] = apply_lim(sp.limiter, uns, false, vcc[i], lrv[i]) - vcc[i];
          }
          // tgrad = tgrad + (s .tens. uLR)  (TENSOR3.f90:283-292)
          double u[3] = {uLR.x, uLR.y, uLR.z};
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) T[i][j] = T[i][j] + s[i] * u[j];
          V3 d = matvec(side == 0 ? LF : RF);
          out[0] = d.x; out[1] = d.y; out[2] = d.z;
        }
        for (int i = 0; i < 3; ++i) (side == 0 ? dL : dR)[2 + i] = out[i];
      }
    }
    for (int v = 0; v < 5; ++v) {
      cell_l[v * nf + f] = prim[v * nc + icl] + dL[v];
      cell_r[v * nf + f] = prim[v * nc + icr] + dR[v];
    }
  }
}

// postlimit_barth.f90:42-223.  A face whose reconstructed increment is exactly zero imposes
// no constraint (the Fortran divides by it; its MAX/MIN of a NaN is compiler-dependent).
void Solver::postlimit_barth(double klim) {
  const int nc = m->ncell, nf = m->nface;
  std::vector<double> ratio(nc);
  auto constrain = [&](int c, double num, double den) {
    if (den == 0.0) return;
    double l = num / den;
    l = std::max(klim * l, 0.0);
    ratio[c] = std::min(ratio[c], l);
  };
  for (int s = 0; s < 2; ++s) {
    std::fill(ratio.begin(), ratio.end(), 1.0);
    for (auto& col : m->colors)  // min is order-independent; a colour's faces touch distinct cells
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < col.size(); ++q) {
      const int f = col[q];
      int icl = m->fc1[f], icr = m->fc2[f];
      double LR = prim[s * nc + icr] - prim[s * nc + icl];
      constrain(icl, LR, cell_l[s * nf + f] - prim[s * nc + icl]);
      constrain(icr, -LR, cell_r[s * nf + f] - prim[s * nc + icr]);
    }
#pragma omp parallel for schedule(static)
    for (int f = 0; f < nf; ++f) {
      int icl = m->fc1[f], icr = m->fc2[f];
      cell_l[s * nf + f] = prim[s * nc + icl] + ratio[icl] * (cell_l[s * nf + f] - prim[s * nc + icl]);
      cell_r[s * nf + f] = prim[s * nc + icr] + ratio[icr] * (cell_r[s * nf + f] - prim[s * nc + icr]);
    }
    for (int c = 0; c < nc; ++c) limratio[s * nc + c] = ratio[c];
  }
  std::fill(ratio.begin(), ratio.end(), 1.0);
  for (auto& col : m->colors)
#pragma omp parallel for schedule(static)
  for (size_t q = 0; q < col.size(); ++q) {
    const int f = col[q];
    int icl = m->fc1[f], icr = m->fc2[f];
    for (int k = 0; k < 3; ++k) {
      double LR = prim[(2 + k) * nc + icr] - prim[(2 + k) * nc + icl];
      constrain(icl, LR, cell_l[(2 + k) * nf + f] - prim[(2 + k) * nc + icl]);
    }
    for (int k = 0; k < 3; ++k) {
      double LR = prim[(2 + k) * nc + icr] - prim[(2 + k) * nc + icl];
      constrain(icr, -LR, cell_r[(2 + k) * nf + f] - prim[(2 + k) * nc + icr]);
    }
  }
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    int icl = m->fc1[f], icr = m->fc2[f];
    for (int k = 0; k < 3; ++k) {
      int v = 2 + k;
      cell_l[v * nf + f] = prim[v * nc + icl] + ratio[icl] * (cell_l[v * nf + f] - prim[v * nc + icl]);
      cell_r[v * nf + f] = prim[v * nc + icr] + ratio[icr] * (cell_r[v * nf + f] - prim[v * nc + icr]);
    }
  }
  for (int c = 0; c < nc; ++c) limratio[2 * nc + c] = ratio[c];
}

// ---------------------------------------------------------------------------
// Face fluxes per unit area, written into flux (5 x nface)
namespace {
struct State { double rho, p; V3 u; };
inline State face_state(const std::vector<double>& q, int nf, int f) {
  State s;
  s.rho = q[f]; s.p = q[nf + f];
  s.u = v3(q[2 * nf + f], q[3 * nf + f], q[4 * nf + f]);
  return s;
}
}  // namespace

// Roe flux-difference splitting (Roe 1981) with Harten's entropy fix on the acoustic waves.
// Typhon parses SCHEME=ROE but has no implementation (calc_flux_inviscid.f90:48-79): this
// is new code written from the published method, with the Roe averages of
// calc_roe_states.f90:35-53.  Fluxes per unit area along the unit normal n.
static void roe_flux(double g, const State& L, const State& R, V3 n, double delta_frac, double* F) {
  const double ig1 = 1.0 / (g - 1.0);
  const double gig1 = g / (g - 1.0);
  // Roe averages (calc_roe_states.f90)
  double t1 = std::sqrt(R.rho / L.rho);
  double rroe = L.rho * t1;
  double kl = 1.0 / (1.0 + t1), kr = t1 * kl;
  V3 uroe = kl * L.u + kr * R.u;
  double hl = gig1 * L.p / L.rho + 0.5 * sqrabs(L.u);
  double hr = gig1 * R.p / R.rho + 0.5 * sqrabs(R.u);
  double hroe = kl * hl + kr * hr;
  double q2 = sqrabs(uroe);
  double a2 = (g - 1.0) * (hroe - 0.5 * q2);
  double a = std::sqrt(a2);
  double vn = dot(uroe, n);
  double vnl = dot(L.u, n), vnr = dot(R.u, n);
  double rel = ig1 * L.p + 0.5 * L.rho * sqrabs(L.u);
  double rer = ig1 * R.p + 0.5 * R.rho * sqrabs(R.u);
  // jumps
  double drho = R.rho - L.rho, dp = R.p - L.p, dvn = vnr - vnl;
  V3 du = R.u - L.u;
  // wave strengths
  double al1 = (dp - rroe * a * dvn) / (2.0 * a2);
  double al5 = (dp + rroe * a * dvn) / (2.0 * a2);
  double al2 = drho - dp / a2;  // entropy wave
  V3 dut = du - dvn * n;        // shear waves (tangential velocity jump)
  // eigenvalues with Harten's fix on the acoustic ones
  double l1 = std::fabs(vn - a), l5 = std::fabs(vn + a), l2 = std::fabs(vn);
  double delta = delta_frac * a;
  if (l1 < delta) l1 = (l1 * l1 + delta * delta) / (2.0 * delta);
  if (l5 < delta) l5 = (l5 * l5 + delta * delta) / (2.0 * delta);
  // dissipation |A| dQ, components (mass, energy, momentum)
  double d_mass = l1 * al1 + l2 * al2 + l5 * al5;
  V3 d_mom = l1 * al1 * (uroe - a * n) + l2 * al2 * uroe + l5 * al5 * (uroe + a * n) +
             (l2 * rroe) * dut;
  double d_ener = l1 * al1 * (hroe - a * vn) + l2 * al2 * (0.5 * q2) + l5 * al5 * (hroe + a * vn) +
                  (l2 * rroe) * (dot(uroe, du) - vn * dvn);
  // central part
  double fl_mass = vnl * L.rho, fr_mass = vnr * R.rho;
  double fl_ener = vnl * (rel + L.p), fr_ener = vnr * (rer + R.p);
  V3 fl_mom = (vnl * L.rho) * L.u + L.p * n, fr_mom = (vnr * R.rho) * R.u + R.p * n;
  F[0] = 0.5 * (fl_mass + fr_mass - d_mass);
  F[1] = 0.5 * (fl_ener + fr_ener - d_ener);
  V3 fm = 0.5 * (fl_mom + fr_mom - d_mom);
  F[2] = fm.x; F[3] = fm.y; F[4] = fm.z;
}

// Test access to the Roe flux on arrays of face states (the property tests of the flux:
// consistency, rotational invariance, contacts).  L, R: [n][5] primitive (rho, p, u, v, w);
// nrm: [n][3] unit normals; F: [n][5] flux per unit area (mass, energy, momentum).
extern "C" int ory_roe_flux(double g, double delta_frac, int n, const double* L, const double* R, const double* nrm,
                            double* F) {
  for (int i = 0; i < n; ++i) {
    const double* l = L + 5 * (size_t)i;
    const double* r = R + 5 * (size_t)i;
    State sl{l[0], l[1], v3(l[2], l[3], l[4])}, sr{r[0], r[1], v3(r[2], r[3], r[4])};
    roe_flux(g, sl, sr, v3(nrm[3 * (size_t)i], nrm[3 * (size_t)i + 1], nrm[3 * (size_t)i + 2]), delta_frac,
             F + 5 * (size_t)i);
  }
  return 0;
}

// calc_jacflux (SOURCE/EQNS/calc_jacflux.f90:49-77): Jacobian of the physical flux along n
// with respect to (rho, rhoE, rhou, rhov, rhow), for one state; row-major 5x5
static void jacflux(double g, const double* st /* rho, p, u, v, w */, V3 fn, double vn, double* J) {
  const double g1 = g - 1.0, ig1 = 1.0 / g1;
  const V3 u = v3(st[2], st[3], st[4]);
  const double v2 = sqrabs(u);
  const double en = ig1 * st[1] / st[0] + .5 * v2;
  for (int k = 0; k < 25; ++k) J[k] = 0.0;
  auto A = [&](int i, int j) -> double& { return J[(i - 1) * 5 + (j - 1)]; };
  A(1, 1) = 0.0; A(1, 2) = 0.0;
  A(1, 3) = fn.x; A(1, 4) = fn.y; A(1, 5) = fn.z;
  A(2, 1) = vn * (g1 * v2 - g * en);
  A(2, 2) = vn * g;
  const double c23 = g * en - .5 * g1 * v2;
  const double t[3] = {fn.x, fn.y, fn.z}, uu[3] = {u.x, u.y, u.z};
  for (int k = 0; k < 3; ++k) A(2, 3 + k) = c23 * t[k] - g1 * vn * uu[k];
  for (int k = 0; k < 3; ++k) A(3 + k, 1) = .5 * g1 * v2 * t[k] - vn * uu[k];
  for (int k = 0; k < 3; ++k) A(3 + k, 2) = g1 * t[k];
  const V3 g1n = g1 * fn;
  const double gn[3] = {g1n.x, g1n.y, g1n.z};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A(3 + i, 3 + j) = uu[i] * t[j] - gn[i] * uu[j];
  A(3, 3) = A(3, 3) + vn;
  A(4, 4) = A(4, 4) + vn;
  A(5, 5) = A(5, 5) + vn;
}

// Wave speeds of the HLLC / HLLE family (calc_flux_hllc.f90:64-124, calc_flux_hlle.f90:64-120):
// beta = 1 or sqrt((g-1)/(2g)) (the B variants); the K variants take the kinetic (EFM)
// estimates cl (m kinw + kind) with m = vn/cl -+ f1 beta, cl = a/f1, f1 = sqrt(g/2),
// kinw = (1 -+ erf(m))/2, kind = -+ exp(-m^2) / (2 sqrt(pi)).  Standard HLLE clamps to 0,
// the kinetic HLLE does not (calc_flux_hlle.f90:110-120).
static void hll_wave_speeds(int scheme, double g, double vnl, double vnr, double al, double ar, double vm, double am,
                            double& sl, double& sr) {
  const bool b = scheme == SCH_HLLCB || scheme == SCH_HLLCKB || scheme == SCH_HLLEB || scheme == SCH_HLLEKB;
  const bool kin = scheme == SCH_HLLCK || scheme == SCH_HLLCKB || scheme == SCH_HLLEK || scheme == SCH_HLLEKB;
  const double beta = b ? std::sqrt((g - 1.0) / (2 * g)) : 1.0;
  if (kin) {
    const double PIcst = 3.141592653589793238462643;
    const double f1 = std::sqrt(0.5 * g), f2 = 0.5 / std::sqrt(PIcst);
    const double cl = al / f1, cr = ar / f1;
    const double modml = vnl / cl - f1 * beta, modmr = vnr / cr + f1 * beta;
    const double kinwl = 0.5 * (1.0 - std::erf(modml)), kinwr = 0.5 * (1.0 + std::erf(modmr));
    const double kindl = -f2 * std::exp(-modml * modml), kindr = +f2 * std::exp(-modmr * modmr);
    sl = std::min(cl * (modml * kinwl + kindl), vm - am);
    sr = std::max(cr * (modmr * kinwr + kindr), vm + am);
  } else if (is_hlle(scheme)) {
    sl = std::min(std::min(0.0, vnl - beta * al), vm - am);
    sr = std::max(std::max(0.0, vnr + beta * ar), vm + am);
  } else {
    sl = std::min(vnl - beta * al, vm - am);
    sr = std::max(vnr + beta * ar, vm + am);
  }
}

void Solver::face_fluxes() {
  const int nf = m->nface;
  const double g = sp.gamma;
  const double ig1 = 1.0 / (g - 1.0);
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    State L = face_state(cell_l, nf, f), R = face_state(cell_r, nf, f);
    V3 fn = m->fnormal[f];
    double F[5];
    if (is_hllc(sp.scheme)) {  // calc_flux_hllc.f90:86-171
      // calc_roe_states.f90:35-53
      const double gig1 = g / (g - 1.0);
      double t1 = std::sqrt(R.rho / L.rho);
      double roe_rho = L.rho * t1;
      double kl = 1.0 / (1.0 + t1);
      double kr = t1 * kl;
      V3 roe_u = kl * L.u + kr * R.u;
      double h1 = gig1 * L.p / L.rho + 0.5 * sqrabs(L.u);
      double h2 = gig1 * R.p / R.rho + 0.5 * sqrabs(R.u);
      h1 = kl * h1 + kr * h2;
      double roe_p = (h1 - 0.5 * sqrabs(roe_u)) * roe_rho / gig1;
      double vnl = dot(L.u, fn), vnr = dot(R.u, fn);
      double al = std::sqrt(g * L.p / L.rho), ar = std::sqrt(g * R.p / R.rho);
      double vm = dot(roe_u, fn);
      double am = std::sqrt(g * roe_p / roe_rho);
      double rel = ig1 * L.p + 0.5 * L.rho * sqrabs(L.u);
      double rer = ig1 * R.p + 0.5 * R.rho * sqrabs(R.u);
      double sl, sr;
      hll_wave_speeds(sp.scheme, g, vnl, vnr, al, ar, vm, am, sl, sr);
      if (calc_jac) {  // calc_flux_hllc.f90:178-203 -> calc_jac_hll.f90:46-57
        double qL[5] = {L.rho, L.p, L.u.x, L.u.y, L.u.z}, qR[5] = {R.rho, R.p, R.u.x, R.u.y, R.u.z};
        double JL[25], JR[25];
        double slc = std::min(sl, 0.0), src = std::max(sr, 0.0);
        jacflux(g, qL, fn, vnl, JL);
        jacflux(g, qR, fn, vnr, JR);
        for (int i = 0; i < 5; ++i) { JL[i * 5 + i] = JL[i * 5 + i] - slc; JR[i * 5 + i] = JR[i * 5 + i] - src; }
        const double cl_ = src / (src - slc), cr_ = -slc / (src - slc);
        for (int k = 0; k < 25; ++k) { jacL[25 * (size_t)f + k] = cl_ * JL[k]; jacR[25 * (size_t)f + k] = cr_ * JR[k]; }
      }
      if (sl >= 0.0) {
        F[0] = vnl * L.rho;
        F[1] = vnl * (rel + L.p);
        V3 mo = (vnl * L.rho) * L.u + L.p * fn;
        F[2] = mo.x; F[3] = mo.y; F[4] = mo.z;
      } else if (sr <= 0.0) {
        F[0] = vnr * R.rho;
        F[1] = vnr * (rer + R.p);
        V3 mo = (vnr * R.rho) * R.u + R.p * fn;
        F[2] = mo.x; F[3] = mo.y; F[4] = mo.z;
      } else {
        double rqL = L.rho * (sl - vnl);
        double rqR = R.rho * (sr - vnr);
        double Sst = (rqR * vnr - rqL * vnl - R.p + L.p) / (rqR - rqL);
        double iks, rst, pst, rest;
        V3 rvst;
        if (Sst >= 0.0) {
          iks = 1.0 / (sl - Sst);
          rst = rqL * iks;
          pst = L.p - rqL * (vnl - Sst);
          rvst = iks * ((rqL * L.u) + (pst - L.p) * fn);
          rest = iks * (rel * (sl - vnl) - L.p * vnl + pst * Sst);
        } else {
          iks = 1.0 / (sr - Sst);
          rst = rqR * iks;
          pst = R.p - rqR * (vnr - Sst);
          rvst = iks * ((rqR * R.u) + (pst - R.p) * fn);
          rest = iks * (rer * (sr - vnr) - R.p * vnr + pst * Sst);
        }
        F[0] = Sst * rst;
        F[1] = Sst * (rest + pst);
        V3 mo = (Sst * rvst) + (pst * fn);
        F[2] = mo.x; F[3] = mo.y; F[4] = mo.z;
      }
    } else if (is_hlle(sp.scheme)) {  // calc_flux_hlle.f90:83-150
      const double gig1 = g / (g - 1.0);
      double t1 = std::sqrt(R.rho / L.rho);  // calc_roe_states.f90:35-53
      double roe_rho = L.rho * t1;
      double kl0 = 1.0 / (1.0 + t1);
      double kr0 = t1 * kl0;
      V3 roe_u = kl0 * L.u + kr0 * R.u;
      double h1 = gig1 * L.p / L.rho + 0.5 * sqrabs(L.u);
      double h2 = gig1 * R.p / R.rho + 0.5 * sqrabs(R.u);
      h1 = kl0 * h1 + kr0 * h2;
      double roe_p = (h1 - 0.5 * sqrabs(roe_u)) * roe_rho / gig1;
      double vnl = dot(L.u, fn), vnr = dot(R.u, fn);
      double al = std::sqrt(g * L.p / L.rho), ar = std::sqrt(g * R.p / R.rho);
      double vm = dot(roe_u, fn);
      double am = std::sqrt(g * roe_p / roe_rho);
      double rel = ig1 * L.p + .5 * L.rho * sqrabs(L.u);
      double rer = ig1 * R.p + .5 * R.rho * sqrabs(R.u);
      double sl, sr;
      hll_wave_speeds(sp.scheme, g, vnl, vnr, al, ar, vm, am, sl, sr);
      double iks = 1.0 / (sr - sl);
      double kl = sr * iks, kr = -sl * iks, ku = sl * sr * iks;
      F[0] = (kl * vnl - ku) * L.rho + (kr * vnr + ku) * R.rho;
      F[1] = (kl * vnl - ku) * rel + (kr * vnr + ku) * rer + (kl * vnl * L.p + kr * vnr * R.p);
      V3 mo = ((kl * vnl - ku) * L.rho) * L.u + ((kr * vnr + ku) * R.rho) * R.u + (kl * L.p + kr * R.p) * fn;
      F[2] = mo.x; F[3] = mo.y; F[4] = mo.z;
      if (calc_jac) {  // calc_jac_hll.f90:46-57 with the flux's wave speeds
        double qL[5] = {L.rho, L.p, L.u.x, L.u.y, L.u.z}, qR[5] = {R.rho, R.p, R.u.x, R.u.y, R.u.z};
        double JL[25], JR[25];
        jacflux(g, qL, fn, vnl, JL);
        jacflux(g, qR, fn, vnr, JR);
        for (int i = 0; i < 5; ++i) { JL[i * 5 + i] = JL[i * 5 + i] - sl; JR[i * 5 + i] = JR[i * 5 + i] - sr; }
        const double cl_ = sr / (sr - sl), cr_ = -sl / (sr - sl);
        for (int k = 0; k < 25; ++k) { jacL[25 * (size_t)f + k] = cl_ * JL[k]; jacR[25 * (size_t)f + k] = cr_ * JR[k]; }
      }
    } else if (sp.scheme == SCH_AUSMM) {  // calc_flux_ausmm.f90:62-118 (no Jacobian in Typhon)
      const double gig1 = g / (g - 1.0);
      const double al = std::sqrt(g * L.p / L.rho), ar = std::sqrt(g * R.p / R.rho);
      const double mnl = dot(L.u, fn) / al, mnr = dot(R.u, fn) / ar;
      double mp, pp, mm, pm;
      if (mnl >= 1.0) { mp = mnl; pp = 1.0; }
      else if (mnl <= -1.0) { mp = 0.0; pp = 0.0; }
      else { mp = .25 * ((mnl + 1.0) * (mnl + 1.0)); pp = mp * (2.0 - mnl); }
      if (mnr <= -1.0) { mm = mnr; pm = 1.0; }
      else if (mnr >= 1.0) { mm = 0.0; pm = 0.0; }
      else { mm = -.25 * ((mnr - 1.0) * (mnr - 1.0)); pm = -mm * (2.0 + mnr); }
      const double ms = mp + mm;
      const double wl = al * std::max(0.0, ms), wr = ar * std::min(0.0, ms);
      const double rhl = gig1 * L.p + .5 * L.rho * sqrabs(L.u);
      const double rhr = gig1 * R.p + .5 * R.rho * sqrabs(R.u);
      F[0] = wl * L.rho + wr * R.rho;
      F[1] = wl * rhl + wr * rhr;
      V3 mo = ((wl * L.rho) * L.u + (wr * R.rho) * R.u) + (pp * L.p + pm * R.p) * fn;
      F[2] = mo.x; F[3] = mo.y; F[4] = mo.z;
    } else if (sp.scheme == SCH_RUSANOV) {  // calc_flux_rusanov.f90:57-83
      double vnl = dot(L.u, fn), vnr = dot(R.u, fn);
      double al = std::sqrt(g * L.p / L.rho), ar = std::sqrt(g * R.p / R.rho);
      double ray = std::max(std::fabs(vnl) + al, std::fabs(vnr) + ar);
      if (calc_jac) {  // calc_jac_rusanov.f90: (A_L + ray I)/2, (A_R - ray I)/2
        double qL[5] = {L.rho, L.p, L.u.x, L.u.y, L.u.z}, qR[5] = {R.rho, R.p, R.u.x, R.u.y, R.u.z};
        double JL[25], JR[25];
        jacflux(g, qL, fn, vnl, JL);
        jacflux(g, qR, fn, vnr, JR);
        for (int i = 0; i < 5; ++i) { JL[i * 5 + i] = JL[i * 5 + i] + ray; JR[i * 5 + i] = JR[i * 5 + i] - ray; }
        for (int k = 0; k < 25; ++k) { jacL[25 * (size_t)f + k] = .5 * JL[k]; jacR[25 * (size_t)f + k] = .5 * JR[k]; }
      }
      double rel = ig1 * L.p + 0.5 * L.rho * sqrabs(L.u);
      double rer = ig1 * R.p + 0.5 * R.rho * sqrabs(R.u);
      F[0] = 0.5 * ((vnl + ray) * L.rho + (vnr - ray) * R.rho);
      F[1] = 0.5 * ((vnl + ray) * rel + (vnr - ray) * rer + vnl * L.p + vnr * R.p);
      V3 mo = 0.5 * ((((vnl + ray) * L.rho) * L.u + ((vnr - ray) * R.rho) * R.u) + (L.p + R.p) * fn);
      F[2] = mo.x; F[3] = mo.y; F[4] = mo.z;
    } else {
      roe_flux(g, L, R, fn, sp.roe_entropy_fix, F);
      if (calc_jac) {  // new: HLL Jacobian with Davis-Einfeldt wave speeds from the Roe average
        double t1 = std::sqrt(R.rho / L.rho);
        double kl = 1.0 / (1.0 + t1), kr = t1 * kl;
        V3 ur = kl * L.u + kr * R.u;
        double hl = g / (g - 1.0) * L.p / L.rho + 0.5 * sqrabs(L.u);
        double hr = g / (g - 1.0) * R.p / R.rho + 0.5 * sqrabs(R.u);
        double am = std::sqrt((g - 1.0) * (kl * hl + kr * hr - 0.5 * sqrabs(ur)));
        double vm = dot(ur, fn), vnl = dot(L.u, fn), vnr = dot(R.u, fn);
        double al = std::sqrt(g * L.p / L.rho), ar = std::sqrt(g * R.p / R.rho);
        double sl = std::min(std::min(vnl - al, vm - am), 0.0), sr = std::max(std::max(vnr + ar, vm + am), 0.0);
        double qL[5] = {L.rho, L.p, L.u.x, L.u.y, L.u.z}, qR[5] = {R.rho, R.p, R.u.x, R.u.y, R.u.z};
        double JL[25], JR[25];
        jacflux(g, qL, fn, vnl, JL);
        jacflux(g, qR, fn, vnr, JR);
        for (int i = 0; i < 5; ++i) { JL[i * 5 + i] = JL[i * 5 + i] - sl; JR[i * 5 + i] = JR[i * 5 + i] - sr; }
        const double cl_ = sr / (sr - sl), cr_ = -sl / (sr - sl);
        for (int k = 0; k < 25; ++k) { jacL[25 * (size_t)f + k] = cl_ * JL[k]; jacR[25 * (size_t)f + k] = cr_ * JR[k]; }
      }
    }
    for (int v = 0; v < 5; ++v) flux[v * nf + f] = F[v];
  }
}


// calc_viscosity (SOURCE/EQNS/EQNS.f90:225-265)
double Solver::viscosity(double rho, double T) const {
  if (sp.visc_law == 0) return sp.visc_kin * rho;
  const double mu0 = 0.0000168, T0 = 273.00, S = 110.50;  // AIR (def_model_ns.f90:170-173)
  return mu0 * std::pow(T / T0, 1.5) * (T0 + S) / (T + S);
}

// calc_flux_viscous_cell (SOURCE/EQNS/calc_flux_viscous_cell.f90:71-144) on cell states and
// cell gradients (integration_ns_ust.f90:139-159), added to the inviscid flux of every face;
// face gradients from interp_facegradient_vect (SOURCE/MESH/interpface_gradient_vect.f90:59-81)
// and interp_facegradn_scal (SOURCE/MESH/interpface_gradn_scal.f90:60-90), theta = 1.
void Solver::viscous_fluxes() {
  const int nc = m->ncell, nf = m->nface;
  const double r = sp.rgas;
  const double cp = sp.gamma * r / (sp.gamma - 1.0);
  const double theta = 1.0;
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    const int icl = m->fc1[f], icr = m->fc2[f];
    const V3 F = m->fcentre[f], CL = m->ccentre[icl], CR = m->ccentre[icr], n = m->fnormal[f];
    double dHL = vabs(F - CL), dHR = vabs(F - CR);
    const double id = 1.0 / (dHL + dHR);
    dHL = id * dHL;
    dHR = id * dHR;
    const V3 vLR = CR - CL;
    const V3 vL = v3(prim[2 * nc + icl], prim[3 * nc + icl], prim[4 * nc + icl]);
    const V3 vR = v3(prim[2 * nc + icr], prim[3 * nc + icr], prim[4 * nc + icr]);
    const V3 velH = dHR * vL + dHL * vR;
    const double rL = prim[icl], rR = prim[icr], pL = prim[nc + icl], pR = prim[nc + icr];
    const double TL = pL / (rL * r), TR = pR / (rR * r);
    const double TH = dHR * TL + dHL * TR;
    const double rhoH = dHR * rL + dHL * rR;
    auto gv = [&](int c, int k) { return v3(grad[(3 * k) * (size_t)nc + c], grad[(3 * k + 1) * (size_t)nc + c],
                                            grad[(3 * k + 2) * (size_t)nc + c]); };
    const V3 gTL = (1.0 / (rL * r)) * gv(icl, 1) - (pL / ((rL * rL) * r)) * gv(icl, 0);
    const V3 gTR = (1.0 / (rR * r)) * gv(icr, 1) - (pR / ((rR * rR) * r)) * gv(icr, 0);
    const double mu = viscosity(rhoH, TH);
    // face velocity gradient T(i,j) = du_i/dx_j
    double GL[3][3], GR[3][3], G[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        GL[i][j] = grad[(6 + 3 * i + j) * (size_t)nc + icl];
        GR[i][j] = grad[(6 + 3 * i + j) * (size_t)nc + icr];
        G[i][j] = dHL * GR[i][j] + dHR * GL[i][j];
      }
    double gTH;
    if (sp.viscous == VISC_CELLFULL) {
      const double dLR2 = sqrabs(vLR);
      double qL[3] = {vL.x, vL.y, vL.z}, qR[3] = {vR.x, vR.y, vR.z}, w[3] = {vLR.x, vLR.y, vLR.z};
      const V3 e = (theta / dLR2) * vLR;
      double ev[3] = {e.x, e.y, e.z};
      double Fav[3];
      for (int i = 0; i < 3; ++i) Fav[i] = qR[i] - qL[i] - (G[i][0] * w[0] + G[i][1] * w[1] + G[i][2] * w[2]);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) G[i][j] = G[i][j] + Fav[i] * ev[j];
      const double pscal = dot(vLR, n) / dLR2;
      const double Fcomp = pscal * (TR - TL);
      const V3 vi = n - (theta * pscal) * vLR;
      const double Favg = dot(dHL * gTR + dHR * gTL, vi);
      gTH = theta * Fcomp + Favg;
    } else {
      gTH = dot(dHL * gTR + dHR * gTL, n);
    }
    // sigma = mu (G + G^T - 2/3 tr(G) I)
    double Sg[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Sg[i][j] = G[i][j] + G[j][i];
    const double addvisc = -(2.0 / 3.0) * (G[0][0] + G[1][1] + G[2][2]);
    for (int i = 0; i < 3; ++i) Sg[i][i] = Sg[i][i] + addvisc;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Sg[i][j] = mu * Sg[i][j];
    const V3 sn = v3(Sg[0][0] * n.x + Sg[0][1] * n.y + Sg[0][2] * n.z, Sg[1][0] * n.x + Sg[1][1] * n.y + Sg[1][2] * n.z,
                     Sg[2][0] * n.x + Sg[2][1] * n.y + Sg[2][2] * n.z);
    const double svn = dot(sn, velH);
    flux[2 * nf + f] = flux[2 * nf + f] - sn.x;
    flux[3 * nf + f] = flux[3 * nf + f] - sn.y;
    flux[4 * nf + f] = flux[4 * nf + f] - sn.z;
    flux[nf + f] = flux[nf + f] - svn;
    const double conduct = mu * cp / sp.prandtl;
    flux[nf + f] = flux[nf + f] - conduct * gTH;
    if (calc_jac) {  // calc_flux_viscous_cell.f90:149-158
      double idj = mu / (dHR * rL + dHL * rR) / vabs(CR - CL);
      for (int i = 0; i < 5; ++i) {
        jacR[25 * (size_t)f + i * 5 + i] = jacR[25 * (size_t)f + i * 5 + i] - idj;
        jacL[25 * (size_t)f + i * 5 + i] = jacL[25 * (size_t)f + i * 5 + i] + idj;
      }
    }
  }
}

// ns_bocoflux (SOURCE/EQNS/ns_bocoflux.f90:47-111): on adiabatic-wall faces the heat flux is
// replaced by the prescribed one (zero): the conduction term is added back
void Solver::ns_bocoflux() {
  const int nc = m->ncell, nf = m->nface;
  const double r = sp.rgas;
  const double cp = sp.gamma * r / (sp.gamma - 1.0);
  for (auto& b : m->bocos) {
    if (b.kind != BC_WALL && b.kind != BC_NOSLIP) continue;
    for (int f : b.iface) {
      const int icl = m->fc1[f], icr = m->fc2[f];
      const V3 F = m->fcentre[f], CL = m->ccentre[icl], CR = m->ccentre[icr], n = m->fnormal[f];
      double dHL = vabs(F - CL), dHR = vabs(F - CR);
      const double id = 1.0 / (dHL + dHR);
      dHL = id * dHL;
      dHR = id * dHR;
      const V3 vLR = CR - CL;
      const double rL = prim[icl], rR = prim[icr], pL = prim[nc + icl], pR = prim[nc + icr];
      const double TL = pL / (rL * r), TR = pR / (rR * r);
      const double TH = dHR * TL + dHL * TR;
      const double rhoH = dHR * rL + dHL * rR;
      auto gv = [&](int c, int k) { return v3(grad[(3 * k) * (size_t)nc + c], grad[(3 * k + 1) * (size_t)nc + c],
                                              grad[(3 * k + 2) * (size_t)nc + c]); };
      const V3 gTL = (1.0 / (rL * r)) * gv(icl, 1) - (pL / ((rL * rL) * r)) * gv(icl, 0);
      const V3 gTR = (1.0 / (rR * r)) * gv(icr, 1) - (pR / ((rR * rR) * r)) * gv(icr, 0);
      const double mu = viscosity(rhoH, TH);
      double gTH;
      if (sp.viscous == VISC_CELLFULL) {
        const double dLR2 = sqrabs(vLR);
        const double pscal = dot(vLR, n) / dLR2;
        const double Fcomp = pscal * (TR - TL);
        const V3 vi = n - (1.0 * pscal) * vLR;
        gTH = 1.0 * Fcomp + dot(dHL * gTR + dHR * gTL, vi);
      } else {
        gTH = dot(dHL * gTR + dHR * gTL, n);
      }
      const double conduct = mu * cp / sp.prandtl;
      flux[nf + f] = flux[nf + f] + conduct * gTH + 0.0;
    }
  }
}

// flux_to_res.f90:47-144: F *= S, colour-ordered scatter, R *= dtloc/V (interior cells)
void Solver::flux_to_res() {
  const int nc = m->ncell, nci = m->ncell_int, nf = m->nface;
#pragma omp parallel for schedule(static)
  for (int f = 0; f < nf; ++f) {
    for (int v = 0; v < 5; ++v) flux[v * nf + f] = m->fsurf[f] * flux[v * nf + f];
    if (calc_jac)
      for (int k = 0; k < 25; ++k) {
        jacL[25 * (size_t)f + k] = m->fsurf[f] * jacL[25 * (size_t)f + k];
        jacR[25 * (size_t)f + k] = m->fsurf[f] * jacR[25 * (size_t)f + k];
      }
  }
  std::fill(residu.begin(), residu.end(), 0.0);
  for (auto& col : m->colors)  // faces of one colour touch distinct cells
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < col.size(); ++q) {
      const int f = col[q];
      int i1 = m->fc1[f], i2 = m->fc2[f];
      for (int v = 0; v < 5; ++v) {
        residu[v * nc + i1] = residu[v * nc + i1] - flux[v * nf + f];
        residu[v * nc + i2] = residu[v * nc + i2] + flux[v * nf + f];
      }
    }
#pragma omp parallel for schedule(static)
  for (int c = 0; c < nci; ++c) {
    double coef = dtloc[c] / m->cvol[c];
    for (int v = 0; v < 5; ++v) residu[v * nc + c] = coef * residu[v * nc + c];
  }
}


// init_implicit_bdlu.f90:37-49 + build_implicit_bdlu.f90:44-83: row-major 5x5 blocks
void Solver::build_implicit_bdlu() {
  const int nc = m->ncell, nci = m->ncell_int, nf = m->nface, nfi = m->nface_int;
  bdiag.assign(25 * (size_t)nc, 0.0);
  bupper.assign(25 * (size_t)nf, 0.0);
  blower.assign(25 * (size_t)nf, 0.0);
  for (int c = 0; c < nci; ++c)
    for (int i = 0; i < 5; ++i) bdiag[25 * (size_t)c + i * 5 + i] = 1.0;
  for (int f = 0; f < nfi; ++f) {
    const int c1 = m->fc1[f], c2 = m->fc2[f];
    for (int k = 0; k < 25; ++k) {
      bdiag[25 * (size_t)c1 + k] = bdiag[25 * (size_t)c1 + k] + jacL[25 * (size_t)f + k] * dtloc[c1] / m->cvol[c1];
      bupper[25 * (size_t)f + k] = +jacR[25 * (size_t)f + k] * dtloc[c1] / m->cvol[c1];
      bdiag[25 * (size_t)c2 + k] = bdiag[25 * (size_t)c2 + k] - jacR[25 * (size_t)f + k] * dtloc[c2] / m->cvol[c2];
      blower[25 * (size_t)f + k] = -jacL[25 * (size_t)f + k] * dtloc[c2] / m->cvol[c2];
    }
  }
  for (int f = nfi; f < nf; ++f) {
    const int c1 = m->fc1[f], c2 = m->fc2[f];
    for (int k = 0; k < 25; ++k) {
      bdiag[25 * (size_t)c1 + k] = bdiag[25 * (size_t)c1 + k] + jacL[25 * (size_t)f + k] * dtloc[c1] / m->cvol[c1];
      bupper[25 * (size_t)f + k] = +jacR[25 * (size_t)f + k] * dtloc[c1] / m->cvol[c1];
    }
    for (int k = 0; k < 25; ++k) bdiag[25 * (size_t)c2 + k] = 0.0;
    for (int i = 0; i < 5; ++i) bdiag[25 * (size_t)c2 + i * 5 + i] = 1.0;
    for (int k = 0; k < 25; ++k) blower[25 * (size_t)f + k] = 0.0;
  }
}

static inline void matvec5(const double* A, const double* x, double* y) {  // matmul(A, x)
  for (int i = 0; i < 5; ++i) {
    double s = 0.0;
    for (int j = 0; j < 5; ++j) s = s + A[i * 5 + j] * x[j];
    y[i] = s;
  }
}

// SPMAT_BDLU.f90:139-157 (bdlu_yeqax): y = A x, diagonal blocks first, then faces in order
void Solver::bdlu_yeqax(const double* x, double* y) const {
  const int nc = m->ncell, nf = m->nface;
  double t[5];
  for (int c = 0; c < nc; ++c) matvec5(&bdiag[25 * (size_t)c], &x[5 * (size_t)c], &y[5 * (size_t)c]);
  for (int f = 0; f < nf; ++f) {
    const int c1 = m->fc1[f], c2 = m->fc2[f];
    matvec5(&blower[25 * (size_t)f], &x[5 * (size_t)c1], t);
    for (int i = 0; i < 5; ++i) y[5 * (size_t)c2 + i] = y[5 * (size_t)c2 + i] + t[i];
    matvec5(&bupper[25 * (size_t)f], &x[5 * (size_t)c2], t);
    for (int i = 0; i < 5; ++i) y[5 * (size_t)c1 + i] = y[5 * (size_t)c1 + i] + t[i];
  }
}

// SPMAT_BDLU.f90:240-262 (bdlu_yeqmaxpz): y = z - A x
void Solver::bdlu_yeqmaxpz(const double* x, const double* z, double* y) const {
  const int nc = m->ncell, nf = m->nface;
  double t[5];
  for (int c = 0; c < nc; ++c) {
    matvec5(&bdiag[25 * (size_t)c], &x[5 * (size_t)c], t);
    for (int i = 0; i < 5; ++i) y[5 * (size_t)c + i] = z[5 * (size_t)c + i] - t[i];
  }
  for (int f = 0; f < nf; ++f) {
    const int c1 = m->fc1[f], c2 = m->fc2[f];
    matvec5(&blower[25 * (size_t)f], &x[5 * (size_t)c1], t);
    for (int i = 0; i < 5; ++i) y[5 * (size_t)c2 + i] = y[5 * (size_t)c2 + i] - t[i];
    matvec5(&bupper[25 * (size_t)f], &x[5 * (size_t)c2], t);
    for (int i = 0; i < 5; ++i) y[5 * (size_t)c1 + i] = y[5 * (size_t)c1 + i] - t[i];
  }
}

static double dotp(const std::vector<double>& a, const std::vector<double>& b, size_t n) {
  double s = 0.0;  // dot_product, sequential
  for (size_t i = 0; i < n; ++i) s = s + a[i] * b[i];
  return s;
}

// bdlu_gmres (SOURCE/MATH/bdlu_gmres.f90:50-217): restarted GMRES, modified Gram-Schmidt,
// Givens rotations, x0 = b / diag, stop when |r|/|b| < INV_RES * |x0|_1, at most 2*max_it
// restarts.  Returns the number of restarts - 1 (info), or -1 if not converged.
// bdlu_bicgstab.f90:40-80 over all cells (ghost rows are identity with a zero right-hand side)
int Solver::bdlu_bicgstab(double* sol) {
  const size_t dim = 5 * (size_t)m->ncell;
  std::vector<double> r1(dim), r2(dim), p(dim), s(dim), t(dim), v(dim);
  auto dotv = [&](const std::vector<double>& a, const std::vector<double>& b) {
    double x = 0.0;
    for (size_t i = 0; i < dim; ++i) x = x + a[i] * b[i];
    return x;
  };
  for (size_t i = 0; i < dim; ++i) p[i] = sol[i];
  for (int c = 0; c < m->ncell; ++c)
    for (int b = 0; b < 5; ++b) sol[5 * (size_t)c + b] = p[5 * (size_t)c + b] / bdiag[25 * (size_t)c + b * 5 + b];
  double ref = 0.0;
  for (size_t i = 0; i < dim; ++i) ref = ref + std::fabs(sol[i]);
  bdlu_yeqmaxpz(sol, p.data(), r1.data());
  r2 = r1;
  double err = std::numeric_limits<double>::max(), rho0 = 0.0, rho1, beta, alpha = 0.0, omega = 0.0;
  int nit = 0;
  while (err >= ref * inv_res && nit <= imp_max_it) {
    rho1 = dotv(r1, r2);
    if (nit == 0) {
      p = r1;
    } else {
      beta = (rho1 / rho0) * (alpha / omega);
      for (size_t i = 0; i < dim; ++i) p[i] = p[i] - omega * v[i];
      for (size_t i = 0; i < dim; ++i) p[i] = r1[i] + beta * p[i];
    }
    bdlu_yeqax(p.data(), v.data());
    alpha = rho1 / dotv(r2, v);
    for (size_t i = 0; i < dim; ++i) s[i] = r1[i] - alpha * v[i];
    bdlu_yeqax(s.data(), t.data());
    double tt = 0.0;
    for (size_t i = 0; i < dim; ++i) tt = tt + t[i] * t[i];
    omega = dotv(t, s) / tt;
    err = 0.0;
    for (size_t i = 0; i < dim; ++i) err = err + std::fabs(alpha * p[i] + omega * s[i]);
    for (size_t i = 0; i < dim; ++i) sol[i] = sol[i] + alpha * p[i] + omega * s[i];
    for (size_t i = 0; i < dim; ++i) r1[i] = s[i] - omega * t[i];
    rho0 = rho1;
    ++nit;
  }
  gmres_iters = nit;
  return nit <= imp_max_it ? nit - 1 : -1;
}

int Solver::bdlu_gmres(double* sol) {
  const size_t dim = 5 * (size_t)m->ncell;
  const int nk = nkrylov;
  std::vector<double> qc(nk), qs(nk), ss(nk + 1), yy(nk), hh((nk + 1) * (size_t)nk);
  auto H = [&](int i, int j) -> double& { return hh[(size_t)(i - 1) * nk + (j - 1)]; };
  std::vector<double> r1(dim), p1(dim);
  std::vector<std::vector<double>> w1(nk, std::vector<double>(dim)), v1(nk, std::vector<double>(dim));
  for (size_t i = 0; i < dim; ++i) p1[i] = sol[i];
  for (int c = 0; c < m->ncell; ++c)
    for (int b = 0; b < 5; ++b) sol[5 * (size_t)c + b] = p1[5 * (size_t)c + b] / bdiag[25 * (size_t)c + b * 5 + b];
  double ref = 0.0;
  for (size_t i = 0; i < dim; ++i) ref = ref + std::fabs(sol[i]);
  const double normp1 = std::sqrt(dotp(p1, p1, dim));
  const double eps = std::numeric_limits<double>::epsilon();
  double errgmres = std::numeric_limits<double>::max();
  int nit = 0;
  while (errgmres >= ref * inv_res && nit <= imp_max_it * 2) {
    bdlu_yeqmaxpz(sol, p1.data(), r1.data());
    double beta = std::sqrt(dotp(r1, r1, dim));
    double fact = 1.0 / beta;
    for (size_t i = 0; i < dim; ++i) v1[0][i] = fact * r1[i];
    std::fill(ss.begin(), ss.end(), 0.0);
    ss[0] = beta;
    std::fill(hh.begin(), hh.end(), 0.0);
    int jk;
    for (jk = 1; jk <= nk; ++jk) {
      bdlu_yeqax(v1[jk - 1].data(), w1[jk - 1].data());
      for (int ik = 1; ik <= jk; ++ik) {
        H(ik, jk) = dotp(w1[jk - 1], v1[ik - 1], dim);
        for (size_t i = 0; i < dim; ++i) w1[jk - 1][i] = w1[jk - 1][i] - H(ik, jk) * v1[ik - 1][i];
      }
      H(jk + 1, jk) = std::sqrt(dotp(w1[jk - 1], w1[jk - 1], dim));
      for (int ik = 1; ik <= jk - 1; ++ik) {
        double tmp = H(ik, jk);
        H(ik, jk) = qc[ik - 1] * tmp + qs[ik - 1] * H(ik + 1, jk);
        H(ik + 1, jk) = -qs[ik - 1] * tmp + qc[ik - 1] * H(ik + 1, jk);
      }
      if (H(jk + 1, jk) > eps * 10 * normp1) {
        if (jk < nk) {
          fact = 1.0 / H(jk + 1, jk);
          for (size_t i = 0; i < dim; ++i) v1[jk][i] = fact * w1[jk - 1][i];
        }
        if (H(jk, jk) == 0) break;
        double tmp = std::sqrt(H(jk, jk) * H(jk, jk) + H(jk + 1, jk) * H(jk + 1, jk));
        qc[jk - 1] = H(jk, jk) / tmp;
        qs[jk - 1] = H(jk + 1, jk) / tmp;
        H(jk, jk) = tmp;
        H(jk + 1, jk) = 0.0;
        ss[jk] = -qs[jk - 1] * ss[jk - 1];
        ss[jk - 1] = qc[jk - 1] * ss[jk - 1];
        if (std::fabs(ss[jk]) < inv_res * std::fabs(ss[0])) break;
      } else {
        break;
      }
    }
    const int nkk = std::min(jk, nk);
    for (int j = nkk; j >= 1; --j) {
      double tmp = ss[j - 1];
      for (int ik = j + 1; ik <= nkk; ++ik) tmp = tmp - H(j, ik) * yy[ik - 1];
      yy[j - 1] = tmp / H(j, j);
      for (size_t i = 0; i < dim; ++i) sol[i] = sol[i] + yy[j - 1] * v1[j - 1][i];
    }
    bdlu_yeqmaxpz(sol, p1.data(), r1.data());
    ss[nkk] = std::sqrt(dotp(r1, r1, dim));
    errgmres = ss[nkk] / normp1;
    nit = nit + 1;
  }
  gmres_iters = nit;
  return nit <= imp_max_it ? nit - 1 : -1;
}

// calc_rhs with the implicit method (calc_rhs.f90:121-138) then update_field (U += dU):
// steady backward Euler with the stability time step at CFL (global minimum or local)
int Solver::implicit_step(double cfl_, bool local_dt, double* l1) {
  cfl = cfl_;
  double dt = timestep();
  if (!(dt > 0.0)) return -2;
  const int nc = m->ncell, nci = m->ncell_int;
  if (!local_dt) std::fill(dtloc.begin(), dtloc.begin() + nci, dt);
  calc_jac = true;
  jacL.assign(25 * (size_t)m->nface, 0.0);
  jacR.assign(25 * (size_t)m->nface, 0.0);
  calc_rhs();
  calc_jac = false;
  build_implicit_bdlu();
  for (int v = 0; v < 5; ++v)  // build_implicit.f90:66-74: ghost rows of the RHS are zero
    for (int c = nci; c < nc; ++c) residu[v * (size_t)nc + c] = 0.0;
  // packst (implicit_solve.f90:40): per cell (rho, rhoE, rhou, rhov, rhow)
  std::vector<double> x(5 * (size_t)nc);
  for (int c = 0; c < nc; ++c)
    for (int v = 0; v < 5; ++v) x[5 * (size_t)c + v] = residu[v * (size_t)nc + c];
  rhs_b = x;
  int info = inversion == 1 ? bdlu_bicgstab(x.data()) : bdlu_gmres(x.data());
  for (int c = 0; c < nc; ++c)
    for (int v = 0; v < 5; ++v) residu[v * (size_t)nc + c] = x[5 * (size_t)c + v];
  for (size_t k = 0; k < cons.size(); ++k) cons[k] = cons[k] + residu[k];  // update_field.f90:38
  if (l1)
    for (int v = 0; v < 5; ++v) {
      double a = 0.0;
      for (int c = 0; c < nci; ++c) a += std::fabs(residu[v * (size_t)nc + c]);
      l1[v] = a;
    }
  return info;
}

// calc_rhs.f90 explicit part: prim, ghost states, gradient, face states, fluxes, residual
void Solver::calc_rhs() {
  varprim();
  if (sp.gradmeth != GRAD_NONE) {
    boco_cell_state();
    calc_gradient();
    boco_cell_grad();
  }
  hres_states();
  if (sp.postlim == POSTLIM_BARTH) postlimit_barth(0.5);
  if (sp.postlim == POSTLIM_SUPERBARTH) postlimit_barth(1.0);
  boco_face_state();
  face_fluxes();
  if (sp.viscous != VISC_NONE) {
    viscous_fluxes();
    ns_bocoflux();
  }
  if (calc_jac) ns_bocojacobian();
  flux_to_res();
}

// ns_bocojacobian.f90:47-85: on symmetry faces the ghost state is the mirrored cell state, so
// J_L += J_R dQr/dQl with dQr/dQl = I - 2 n n^T on the momentum block, and J_R = 0.
// Other boundary kinds (periodic, wall) keep their Jacobians.
void Solver::ns_bocojacobian() {
  const int nf = m->nface;
  for (const Boco& b : m->bocos) {
    if (b.kind == BC_FARFIELD || b.kind == BC_NOSLIP) {
      for (int f : b.iface) {
        double ql[5];
        for (int v = 0; v < 5; ++v) ql[v] = cell_l[v * (size_t)nf + f];
        double M[25];
        if (b.kind == BC_NOSLIP) noslip_jacobian(b.wall_velocity, M);
        else if (!farfield_jacobian(sp.gamma, sp.farfield, m->fnormal[f], ql, M)) continue;
        double* JL = &jacL[25 * (size_t)f];
        double* JR = &jacR[25 * (size_t)f];
        for (int i = 0; i < 5; ++i)
          for (int j = 0; j < 5; ++j) {
            double a = 0.0;
            for (int k = 0; k < 5; ++k) a = a + JR[i * 5 + k] * M[k * 5 + j];
            JL[i * 5 + j] = JL[i * 5 + j] + a;
          }
        for (int k = 0; k < 25; ++k) JR[k] = 0.0;
      }
      continue;
    }
    if (b.kind == BC_OUTLET_SUP) {  // ns_bocojacobian.f90: dQr/dQl = I
      for (int f : b.iface) {
        double* JL = &jacL[25 * (size_t)f];
        double* JR = &jacR[25 * (size_t)f];
        for (int k = 0; k < 25; ++k) JL[k] = JL[k] + JR[k];
        for (int k = 0; k < 25; ++k) JR[k] = 0.0;
      }
      continue;
    }
    if (b.kind != BC_SYMMETRY) continue;
    for (int f : b.iface) {
      const V3 n = m->fnormal[f];
      const double nn[3] = {n.x, n.y, n.z};
      double M[25];
      for (int k = 0; k < 25; ++k) M[k] = 0.0;
      for (int i = 0; i < 5; ++i) M[i * 5 + i] = 1.0;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[(2 + i) * 5 + 2 + j] = M[(2 + i) * 5 + 2 + j] - 2.0 * (nn[i] * nn[j]);
      double* JL = &jacL[25 * (size_t)f];
      double* JR = &jacR[25 * (size_t)f];
      for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
          double a = 0.0;
          for (int k = 0; k < 5; ++k) a = a + JR[i * 5 + k] * M[k * 5 + j];
          JL[i * 5 + j] = JL[i * 5 + j] + a;
        }
      for (int k = 0; k < 25; ++k) JR[k] = 0.0;
    }
  }
}

// calc_ns_timestep.f90:52-103 + calc_zonetimestep.f90 min over interior cells
double Solver::timestep() {
  const int nc = m->ncell, nci = m->ncell_int;
  const double gg1 = sp.gamma * (sp.gamma - 1.0);
  std::vector<double> sumS(nci, 0.0);
  for (auto& col : m->colors)
#pragma omp parallel for schedule(static)
    for (size_t q = 0; q < col.size(); ++q) {
      const int f = col[q];
      int i1 = m->fc1[f], i2 = m->fc2[f];
      sumS[i1] = sumS[i1] + m->fsurf[f];
      if (i2 < nci) sumS[i2] = sumS[i2] + m->fsurf[f];
    }
  double dt = std::numeric_limits<double>::max();
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(min : dt) reduction(max : bad)
  for (int c = 0; c < nci; ++c) {
    double d = cfl * 2.0 * m->cvol[c] / sumS[c];
    double irho = 1.0 / cons[c];
    double rv2 = cons[2 * nc + c] * cons[2 * nc + c] + cons[3 * nc + c] * cons[3 * nc + c] +
                 cons[4 * nc + c] * cons[4 * nc + c];
    double a2 = (cons[nc + c] - 0.5 * rv2 * irho) * gg1 * irho;
    if (!(a2 > 0.0)) { bad = 1; continue; }  // negative or NaN internal energy
    d = d / (std::sqrt(rv2) * irho + std::sqrt(a2));
    dtloc[c] = d;
    dt = std::min(dt, d);
  }
  return bad ? -1.0 : dt;
}

// treelevel_rungekutta.f90:48-113 then update_field.f90:38 (U += residu) with a global dt, or
// with the per-cell dtloc of timestep() when local (DTCALC = LOCAL_STABILITY_CONDITION)
void Solver::rk_step(double dt, bool local) {
  const int nc = m->ncell;
  const int n = rk.nstage;
  if (!local) std::fill(dtloc.begin(), dtloc.end(), dt);
  std::vector<double> u0 = cons;
  std::vector<std::vector<double>> rhs(n);
  for (int i = 1; i <= n; ++i) {
    if (i >= 2) {
      cons = u0;
      for (int s = 1; s <= i - 1; ++s) {
        double c = rk.c(i - 1, s);
        const size_t nk = cons.size();
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < nk; ++k) cons[k] = cons[k] + c * rhs[s - 1][k];
      }
    }
    calc_rhs();
    rhs[i - 1] = residu;
  }
  // residu = coef(n,1)*rhs1 + sum coef(n,s)*rhs_s   (scale then xeqxpay)
  const size_t nk = residu.size();
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < nk; ++k) residu[k] = rk.c(n, 1) * rhs[0][k];
  for (int s = 2; s <= n; ++s) {
    double c = rk.c(n, s);
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < nk; ++k) residu[k] = residu[k] + c * rhs[s - 1][k];
  }
  cons = u0;
#pragma omp parallel for schedule(static)
  for (size_t k = 0; k < nk; ++k) cons[k] = cons[k] + residu[k];
  (void)nc;
}

void ns_typhon_steady(Solver& s, const NsSteadyParams& p, NsSteadyOut& out) {
  const UMesh* m = s.m;
  if (p.rk_method >= 0) s.rk = rk_table(p.rk_method);
  const int nc = m->ncell, nci = m->ncell_int, nf = m->nface;
  // calc_refcons.f90 + define_refcons (MENU_SOLVER.f90:260-275)
  double ref0 = 0.0, ref1 = 0.0, totvol = 0.0;
  for (int c = 0; c < nci; ++c) ref0 = ref0 + s.cons[c] * m->cvol[c];
  for (int c = 0; c < nci; ++c) ref1 = ref1 + s.cons[nc + c] * m->cvol[c];
  for (int c = 0; c < nci; ++c) totvol = totvol + m->cvol[c];
  ref0 = ref0 / totvol;
  ref1 = ref1 / totvol;
  const double refv = std::sqrt(ref0 * ref1);
  const double tiny = std::numeric_limits<double>::min();
  double w_ref = 1.0, w_cur = 1.0, z_reforig = 0.0;
  int iters = 0;
  for (int icycle = 1; icycle <= p.max_cycles; ++icycle) {
    const double wcur_res = w_cur, wres_ref = w_ref;
    w_cur = tiny;
    double z_ref = w_cur, z_cur = z_ref;
    const int maxit = p.max_iters - iters;
    int it_loc = 0;
    bool end = false;
    while (!end) {
      ++it_loc;
      ++iters;
      double cfl = p.cfl * std::max(1.0, 1.0 - std::log10(z_cur / z_ref) - std::log10(wcur_res / wres_ref));
      cfl = std::min(cfl, p.cfl_max);
      if (p.rk_method >= 0) {  // explicit: stability time step (calc_zonetimestep.f90:93-117)
        s.cfl = cfl;
        s.rk_step(s.timestep(), p.local_dt);
      } else {
        s.implicit_step(cfl, false, nullptr);
      }
      // update_field.f90:45-60: scalars rho, rho E, then the momentum vector cell by cell
      double a = 0.0, b = 0.0;
      for (int c = 0; c < nci; ++c) a = a + std::fabs(s.residu[c]);
      for (int c = 0; c < nci; ++c) b = b + std::fabs(s.residu[nc + c]);
      z_cur = 0.0 + a / ref0;
      z_cur = z_cur + b / ref1;
      for (int c = 0; c < nci; ++c) {
        const double mx = s.residu[2 * nc + c], my = s.residu[3 * nc + c], mz = s.residu[4 * nc + c];
        z_cur = z_cur + std::sqrt(mx * mx + my * my + mz * mz) / refv;
      }
      z_ref = std::max(z_ref, z_cur);
      if (z_cur / z_ref <= p.cycle_res) end = true;
      if (it_loc == maxit) end = true;
      out.log_res.push_back(std::log10(z_cur));
    }
    if (icycle == 1) z_reforig = z_ref;
    if (z_cur / z_reforig >= w_cur / w_ref) {
      w_cur = z_cur;
      w_ref = z_reforig;
    }
    // integ_ustboco.f90: flux of the last right-hand side, ghost primitive state
    double fs[5] = {0, 0, 0, 0, 0}, qa[5] = {0, 0, 0, 0, 0}, area = 0.0;
    for (int f : p.history_faces) {
      const int g = m->fc2[f];
      const double S = m->fsurf[f];
      for (int v = 0; v < 5; ++v) {
        qa[v] = qa[v] + S * s.prim[v * (size_t)nc + g];
        fs[v] = fs[v] + s.flux[v * (size_t)nf + f];
      }
    }
    for (int f : p.history_faces) area = area + m->fsurf[f];
    for (int v = 0; v < 5; ++v) {
      out.flux_sum.push_back(fs[v]);
      out.ghost_avg.push_back(qa[v] / area);
    }
    out.cycle_end.push_back(iters);
    if (w_cur / w_ref <= p.global_res || iters >= p.max_iters) break;
  }
}

}  // namespace ory
