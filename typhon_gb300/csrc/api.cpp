// C ABI of libtyphon_gpu (declared in include/typhon_gpu.h): handle management, host-side
// precomputation of the static per-face/per-cell data, and the launch order of the
// residual and Runge-Kutta pipelines.  Kernels live in kernels_exact.cu / kernels_fast.cu.
//
// Host arithmetic that feeds the kernels (least-squares factors, reconstruction geometry)
// follows the operation order of Typhon's set-up routines and is compiled without
// floating-point contraction, so the exact mode reproduces Typhon's values bit for bit:
//   least-squares factors   SOURCE/MGRID/precalc_grad_lsq.f90:82-155, SOURCE/MATH/MATRIX.f90:42-70
//   MUSCL geometry          SOURCE/EQNS/hres_ns_musclfast.f90:40-50, hres_ns_muscl.f90:40-50
//   sum of face surfaces    SOURCE/EQNS/calc_ns_timestep.f90:60-73
//   gather order            SOURCE/MAIN/flux_to_res.f90:90-113 (colour by colour)
//   RK stage combination    SOURCE/MAIN/treelevel_rungekutta.f90:60-113, SOURCE/PARAM/MENU_NUM.f90:368-449
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/typhon_gpu.h"
#include "devmesh.hpp"
#include "handle.hpp"
#include "internal.hpp"

using namespace tyk;
using tyi::cuda_fail;
using tyi::pad32;

namespace tyi {
static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
const char* last_error() { return g_last_error.c_str(); }
}  // namespace tyi

namespace {


struct RkTab {
  int n = 0;
  double c[kMaxStage][kMaxStage] = {};  // c[i-1][j-1] = coef(i,j)
};
bool rk_table(int method, RkTab& t) {
  t = RkTab();
  auto row = [&](int i, std::initializer_list<double> v) {
    int j = 0;
    for (double x : v) t.c[i][j++] = x;
  };
  switch (method) {
    case TY_RK_EXPLICIT: t.n = 1; row(0, {1.}); break;  // treelevel_explicit.f90: U += residu
    case TY_RK2: t.n = 2; row(0, {.5}); row(1, {0., 1.}); break;
    case TY_RK2SSP: t.n = 2; row(0, {1.}); row(1, {.5, .5}); break;
    case TY_RK3SSP: t.n = 3; row(0, {1.}); row(1, {.25, .25}); row(2, {1. / 6., 1. / 6., 4. / 6.}); break;
    case TY_RK4: t.n = 4; row(0, {.5}); row(1, {0., .5}); row(2, {0., 0., 1.});
      row(3, {1. / 6., 2. / 6., 2. / 6., 1. / 6.}); break;
    case TY_LSRK25BB: t.n = 5; row(0, {0.1815754863270908}); row(1, {0., 0.238260222208392});
      row(2, {0., 0., 0.330500707328}); row(3, {0., 0., 0., 0.5}); row(4, {0., 0., 0., 0., 1.}); break;
    case TY_LSRK26BB: t.n = 6; row(0, {0.11797990162882}); row(1, {0., 0.18464696649448});
      row(2, {0., 0., 0.24662360430959}); row(3, {0., 0., 0., 0.33183954253762});
      row(4, {0., 0., 0., 0., 0.5}); row(5, {0., 0., 0., 0., 0., 1.}); break;
    case TY_LSRK12BS: t.n = 2; row(0, {1.}); row(1, {0., 1.}); break;
    case TY_LSRK13BS: t.n = 3; row(0, {.15}); row(1, {0., .4}); row(2, {0., 0., 1.}); break;
    default: return false;
  }
  return true;
}

// Per-stage update plans: the state of stage k is u0 + sum_{s<k} coef(k-1,s) rhs_s, built up
// term by term in increasing s as soon as rhs_s is known; the final residual
// sum_s coef(n,s) rhs_s likewise (scale, then x = x + a*y).
void make_plans(const RkTab& t, RkStagePlan* plans) {
  bool started[kMaxStage + 2] = {};
  for (int i = 1; i <= t.n; ++i) {
    RkStagePlan& p = plans[i - 1];
    p = RkStagePlan();
    for (int k = i + 1; k <= t.n; ++k) {
      double c = t.c[k - 2][i - 1];
      bool is_next = (k == i + 1);
      if (c != 0.0 || (is_next)) {
        if (c == 0.0 && is_next && !started[k]) {
          p.ops[p.nops++] = RkOp{k, 1, 1, 0.0};  // next stage state equals u0
        } else if (c != 0.0 || is_next) {
          p.ops[p.nops++] = RkOp{k, started[k] ? 0 : 1, is_next ? 1 : 0, c};
        }
        started[k] = true;
      }
    }
    p.has_acc = 1;
    p.acc_init = (i == 1);
    p.c_acc = t.c[t.n - 1][i - 1];
    p.final_stage = (i == t.n);
  }
}

}  // namespace

namespace {

// least-squares factors for the selected gradient method (precalc_grad_lsq.f90:43-159)
int build_lsq(ty_mesh* h, int gradmeth) {
  DevMesh& m = h->m;
  const int nci = m.nci, nf = m.nf, nfi = m.nfi;
  std::vector<double> dcg(3 * (size_t)m.ldf, 0.0), dpre(3 * (size_t)nf);
  for (int f = 0; f < nf; ++f) {
    const double* a = &h->ccentre[3 * (size_t)h->fc1[f]];
    const double* b = &h->ccentre[3 * (size_t)h->fc2[f]];
    double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
    // precalc: d (LSQ) or d/|d|^2 (W-LSQ); calc_gradient: d or d/|d|^4
    double px = dx, py = dy, pz = dz, gx = dx, gy = dy, gz = dz;
    if (gradmeth == TY_GRAD_LSQW) {
      double s = dx * dx + dy * dy + dz * dz;
      px = dx / s; py = dy / s; pz = dz / s;
      double s2 = s * s;
      gx = dx / s2; gy = dy / s2; gz = dz / s2;
    }
    dpre[3 * (size_t)f] = px; dpre[3 * (size_t)f + 1] = py; dpre[3 * (size_t)f + 2] = pz;
    dcg[f] = gx; dcg[(size_t)m.ldf + f] = gy; dcg[2 * (size_t)m.ldf + f] = gz;
  }
  std::vector<double> A(9 * (size_t)nci, 0.0);  // column-major 3x3 per cell
  auto addm = [&](int c, const double* d) {
    double im[9];
    im[0] = d[0] * d[0]; im[4] = d[1] * d[1]; im[8] = d[2] * d[2];
    im[3] = d[0] * d[1]; im[1] = im[3];
    im[6] = d[0] * d[2]; im[2] = im[6];
    im[7] = d[1] * d[2]; im[5] = im[7];
    for (int k = 0; k < 9; ++k) A[9 * (size_t)c + k] = A[9 * (size_t)c + k] + im[k];
  };
  for (int f = 0; f < nfi; ++f) { addm(h->fc1[f], &dpre[3 * (size_t)f]); addm(h->fc2[f], &dpre[3 * (size_t)f]); }
  for (int f = nfi; f < nf; ++f) addm(h->fc1[f], &dpre[3 * (size_t)f]);
  if (m.dim == 2)
    for (int c = 0; c < nci; ++c) A[9 * (size_t)c + 8] = A[9 * (size_t)c + 8] + 1.0;
  std::vector<double> L(6 * (size_t)nci);
  for (int c = 0; c < nci; ++c) {
    double* a = &A[9 * (size_t)c];
    auto E = [&](int i, int j) -> double& { return a[(j - 1) * 3 + (i - 1)]; };
    for (int i = 1; i <= 3; ++i)
      for (int j = i; j <= 3; ++j) {
        double sum = E(i, j);
        for (int k = i - 1; k >= 1; --k) sum = sum - E(i, k) * E(j, k);
        if (i == j) {
          if (!(sum > 0.0)) {
            tyi::set_error("least-squares matrix not positive definite at cell " + std::to_string(c));
            return TY_ERR_LSQ;
          }
          E(i, i) = std::sqrt(sum);
        } else {
          E(j, i) = sum / E(i, i);
        }
      }
    L[c] = E(1, 1); L[nci + (size_t)c] = E(2, 1); L[2 * (size_t)nci + c] = E(3, 1);
    L[3 * (size_t)nci + c] = E(2, 2); L[4 * (size_t)nci + c] = E(3, 2); L[5 * (size_t)nci + c] = E(3, 3);
  }
  // fast mode: w = A^-1 d per (face, side), so that grad = sum dq * w
  std::vector<double> w(6 * (size_t)m.ldf, 0.0);
  for (int f = 0; f < nf; ++f) {
    for (int side = 0; side < 2; ++side) {
      int c = side ? h->fc2[f] : h->fc1[f];
      if (c >= nci) continue;
      double L11 = L[c], L21 = L[nci + (size_t)c], L31 = L[2 * (size_t)nci + c];
      double L22 = L[3 * (size_t)nci + c], L32 = L[4 * (size_t)nci + c], L33 = L[5 * (size_t)nci + c];
      double x1 = dcg[f], x2 = dcg[(size_t)m.ldf + f], x3 = dcg[2 * (size_t)m.ldf + f];
      x1 = x1 / L11; x2 = (x2 - L21 * x1) / L22; x3 = (x3 - L31 * x1 - L32 * x2) / L33;
      x3 = x3 / L33; x2 = (x2 - L32 * x3) / L22; x1 = (x1 - L21 * x2 - L31 * x3) / L11;
      w[(3 * side) * (size_t)m.ldf + f] = x1;
      w[(3 * side + 1) * (size_t)m.ldf + f] = x2;
      w[(3 * side + 2) * (size_t)m.ldf + f] = x3;
    }
  }
  int rc;
  if ((rc = h->upload(m.dcg, dcg))) return rc;
  if ((rc = h->upload(m.lsq, L))) return rc;
  if ((rc = h->upload(m.lsqw, w))) return rc;
  h->lsq_gradmeth = gradmeth;
  return TY_OK;
}

// MUSCL geometry (hres_ns_musclfast.f90:40-50 / hres_ns_muscl.f90:40-50)
int build_muscl_geometry(ty_mesh* h, int highres) {
  DevMesh& m = h->m;
  const size_t lf = m.ldf;
  std::vector<double> uLR(3 * lf, 0.0), dLR(lf, 1.0), kLF(lf, 0.0), kRF(lf, 0.0), LF(3 * lf, 0.0), RF(3 * lf, 0.0);
  for (int f = 0; f < m.nf; ++f) {
    const double* CL = &h->ccentre[3 * (size_t)h->fc1[f]];
    const double* CR = &h->ccentre[3 * (size_t)h->fc2[f]];
    const double* F = &h->fcentre[3 * (size_t)f];
    double ux = CR[0] - CL[0], uy = CR[1] - CL[1], uz = CR[2] - CL[2];
    double d;
    if (highres == TY_HRES_MUSCLFAST) {
      double a0 = F[0] - CL[0], a1 = F[1] - CL[1], a2 = F[2] - CL[2];
      double b0 = F[0] - CR[0], b1 = F[1] - CR[1], b2 = F[2] - CR[2];
      double kl = std::sqrt(a0 * a0 + a1 * a1 + a2 * a2);
      double kr = -std::sqrt(b0 * b0 + b1 * b1 + b2 * b2);
      d = kl - kr;
      kLF[f] = kl; kRF[f] = kr;
    } else {
      LF[f] = F[0] - CL[0]; LF[lf + f] = F[1] - CL[1]; LF[2 * lf + f] = F[2] - CL[2];
      RF[f] = F[0] - CR[0]; RF[lf + f] = F[1] - CR[1]; RF[2 * lf + f] = F[2] - CR[2];
      d = std::sqrt(ux * ux + uy * uy + uz * uz);
    }
    dLR[f] = d;
    uLR[f] = ux / d; uLR[lf + f] = uy / d; uLR[2 * lf + f] = uz / d;
  }
  // fast mode: 1/dLR and, for MUSCL/-UNS without limiter, the merged weights
  //   increment = grad q . (CF - (u.CF) u) + (q_nb - q_c) (u.CF)/dLR  (sign of the last term
  //   folded in for the fc2 side, whose q_nb - q_c is -(q(fc2) - q(fc1)))
  std::vector<double> inv(lf, 0.0), recw(8 * lf, 0.0);
  for (int f = 0; f < m.nf; ++f) {
    inv[f] = 1.0 / dLR[f];
    if (highres == TY_HRES_MUSCLFAST) continue;
    double u[3] = {uLR[f], uLR[lf + f], uLR[2 * lf + f]};
    for (int side = 0; side < 2; ++side) {
      const std::vector<double>& CF = side ? RF : LF;
      double c[3] = {CF[f], CF[lf + f], CF[2 * lf + f]};
      double uc = u[0] * c[0] + u[1] * c[1] + u[2] * c[2];
      for (int k = 0; k < 3; ++k) recw[(4 * side + k) * lf + f] = c[k] - uc * u[k];
      recw[(4 * side + 3) * lf + f] = (side ? -uc : uc) / dLR[f];
    }
  }
  int rc;
  if ((rc = h->upload(m.uLR, uLR)) || (rc = h->upload(m.dLR, dLR)) || (rc = h->upload(m.kLF, kLF)) ||
      (rc = h->upload(m.kRF, kRF)) || (rc = h->upload(m.LF, LF)) || (rc = h->upload(m.RF, RF)) ||
      (rc = h->upload(m.invdLR, inv)) || (rc = h->upload(m.recw, recw)))
    return rc;
  h->geo_highres = highres;
  return TY_OK;
}

// viscous face geometry (calc_flux_viscous_cell.f90:82-90): HL/(HL+HR), HR/(HL+HR), C_R - C_L
int build_viscous_geometry(ty_mesh* h) {
  DevMesh& m = h->m;
  const size_t lf = m.ldf;
  std::vector<double> g(5 * lf, 0.0);
  for (int f = 0; f < m.nf; ++f) {
    const double* CL = &h->ccentre[3 * (size_t)h->fc1[f]];
    const double* CR = &h->ccentre[3 * (size_t)h->fc2[f]];
    const double* F = &h->fcentre[3 * (size_t)f];
    const double a0 = F[0] - CL[0], a1 = F[1] - CL[1], a2 = F[2] - CL[2];
    const double b0 = F[0] - CR[0], b1 = F[1] - CR[1], b2 = F[2] - CR[2];
    double dHL = std::sqrt(a0 * a0 + a1 * a1 + a2 * a2), dHR = std::sqrt(b0 * b0 + b1 * b1 + b2 * b2);
    const double id = 1.0 / (dHL + dHR);
    dHL = id * dHL;
    dHR = id * dHR;
    g[f] = dHL;
    g[lf + f] = dHR;
    g[2 * lf + f] = CR[0] - CL[0];
    g[3 * lf + f] = CR[1] - CL[1];
    g[4 * lf + f] = CR[2] - CL[2];
  }
  int rc = h->upload(m.vgeo, g);
  if (rc) return rc;
  h->visc_ready = true;
  return TY_OK;
}

}  // namespace

namespace tyi {

int check_err(ty_mesh* h) {
  int e[2] = {0, 0};
  TY_CU(cudaMemcpyAsync(e, h->s.err, 2 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  if (e[0] != 0) {
    TY_CU(cudaMemsetAsync(h->s.err, 0, 4 * sizeof(int), h->stream));
    tyi::set_error(std::string(ty_error_string(e[0])) + " at cell " + std::to_string(e[1]));
    return e[0];
  }
  return TY_OK;
}

int set_dt_slot(ty_mesh* h, int slot, double v) {
  unsigned long long b;
  std::memcpy(&b, &v, 8);
  // pinned staging word per slot keeps the copy asynchronous and ordered on the stream
  unsigned long long* host = reinterpret_cast<unsigned long long*>(h->dtbits_host) + slot;
  *host = b;
  TY_CU(cudaMemcpyAsync(h->s.dtbits + slot, host, 8, cudaMemcpyHostToDevice, h->stream));
  return TY_OK;
}


int ensure_prim(ty_mesh* h) {
  if (h->prim_valid) return TY_OK;
  cudaError_t e = MODE_CALL(h, prim_from, h->m, h->s, h->o, h->s.u0, h->stream, &h->prof);
  if (e != cudaSuccess) return cuda_fail(e, "prim");
  h->prim_valid = true;
  return TY_OK;
}

int ready(ty_mesh* h) {
  if (!h) return TY_ERR_ARG;
  if (!h->has_params || !h->has_state) {
    tyi::set_error("set the parameters and upload a state first");
    return TY_ERR_STATE;
  }
  if (h->heat_bc) {
    tyi::set_error("the mesh has heat-conduction (TY_BC_HEAT) boundaries: no Navier-Stokes boundary state");
    return TY_ERR_UNSUPPORTED;
  }
  if (h->inout_bc && (!h->bcdata_set || !(h->o.rgas > 0.0))) {
    tyi::set_error("inlets / outlets need ty_set_bc_data and ty_spat_params.rgas > 0");
    return TY_ERR_STATE;
  }
  TY_CU(cudaSetDevice(h->device));
  return TY_OK;
}

int stage_faces(ty_mesh* h) {
  // every table a kernel of this configuration reads must exist before any launch
  if ((h->o.viscous != TY_VISC_NONE && !h->m.vgeo) || (h->o.gradmeth != TY_GRAD_NONE && !h->m.lsq) ||
      (h->o.highres != TY_HRES_NONE && !h->m.dLR)) {
    tyi::set_error("internal: a geometry table of the selected scheme is missing");
    return TY_ERR_STATE;
  }
  cudaError_t e = MODE_CALL(h, residual_faces, h->m, h->s, h->o, h->stream, &h->prof);
  if (e != cudaSuccess) return cuda_fail(e, "residual faces");
  return TY_OK;
}

int ensure_lsq(ty_mesh* h) {
  if (h->lsq_gradmeth == TY_GRAD_LSQ) return TY_OK;
  return build_lsq(h, TY_GRAD_LSQ);
}

}  // namespace tyi

using namespace tyi;

namespace {

int ensure_pk(ty_mesh* h, const RkStagePlan* plans, int n) {
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < plans[i].nops; ++k) {
      const RkOp& op = plans[i].ops[k];
      if (!h->s.pk[op.target]) {
        int rc = h->alloc(h->s.pk[op.target], 5 * (size_t)h->m.ldc);
        if (rc) return rc;
      }
    }
  return TY_OK;
}

// one RK step; dt either host value or device slot dtbits_cur.  dtbits_next: where the
// final stage writes the next step's stability time step (or null).
int run_step(ty_mesh* h, const RkTab& t, double dt, const unsigned long long* dtbits_cur,
             unsigned long long* dtbits_next, double cfl, bool store_acc = false,
             const double* dtloc = nullptr) {
  RkStagePlan plans[kMaxStage];
  make_plans(t, plans);
  plans[t.n - 1].store_acc = store_acc ? 1 : 0;
  for (int i = 0; i < t.n; ++i) plans[i].dtloc = dtloc;
  int rc = ensure_pk(h, plans, t.n);
  if (rc) return rc;
  rc = ensure_prim(h);
  if (rc) return rc;
  for (int i = 0; i < t.n; ++i) {
    if ((rc = stage_faces(h))) return rc;
    if (h->ghost_rows) {
      GhostRk r;
      r.stage = i;
      r.nstage = t.n;
      for (int s = 0; s < i; ++s) r.cs[s] = t.c[i - 1][s];
      for (int s = 0; s < t.n; ++s) r.cf[s] = t.c[t.n - 1][s];
      cudaError_t e = MODE_CALL(h, ghost_rows, h->m, h->s, h->o, r, h->gcons, h->gres, h->gprim, h->stream);
      if (e != cudaSuccess) return cuda_fail(e, "ghost rows");
    }
    cudaError_t e = MODE_CALL(h, rk_update, h->m, h->s, h->o, plans[i], dt, dtbits_cur,
                              i == t.n - 1 ? dtbits_next : nullptr, cfl, h->stream, &h->prof);
    if (e != cudaSuccess) return cuda_fail(e, "rk update");
  }
  h->prim_valid = true;  // the final update wrote the primitive variables of u0
  return TY_OK;
}

}  // namespace

extern "C" {

const char* ty_version(void) { return "typhon_gb300 0.1 (sm_103a)"; }

const char* ty_error_string(int st) {
  switch (st) {
    case TY_OK: return "ok";
    case TY_ERR_ARG: return "invalid argument";
    case TY_ERR_CUDA: return "CUDA error";
    case TY_ERR_NOMEM: return "device allocation failed";
    case TY_ERR_MESH: return "inconsistent mesh";
    case TY_ERR_NEGENERGY: return "negative or NaN internal energy";
    case TY_ERR_NANDT: return "NaN time step";
    case TY_ERR_STATE: return "call out of order";
    case TY_ERR_UNSUPPORTED: return "unsupported option";
    case TY_ERR_LSQ: return "least-squares matrix not positive definite";
  }
  return "unknown status";
}

const char* ty_last_error(void) { return tyi::last_error(); }

int ty_mesh_create(const ty_mesh_desc* d, int device, ty_mesh** out) {
  if (!d || !out) return TY_ERR_ARG;
  *out = nullptr;
  const int nci = d->ncell_int, nc = d->ncell, nfi = d->nface_int, nf = d->nface;
  if ((d->dim != 2 && d->dim != 3) || nci <= 0 || nc < nci || nfi < 0 || nf < nfi || nc - nci != nf - nfi ||
      !d->facecell || !d->face_normal || !d->face_surface || !d->face_centre || !d->cell_centre ||
      !d->cell_volume || !d->face_color || !d->face_bc || !d->face_partner) {
    tyi::set_error("ty_mesh_desc: missing array or inconsistent sizes");
    return TY_ERR_ARG;
  }
  int ndev = 0;
  TY_CU(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(device));
  ty_mesh* h = new ty_mesh();
  auto bail = [&](int rc) { ty_mesh_destroy(h); return rc; };
  h->device = device;
  if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) return bail(TY_ERR_CUDA);
  h->stream = h->own_stream;
  DevMesh& m = h->m;
  m.dim = d->dim; m.nci = nci; m.nc = nc; m.nfi = nfi; m.nf = nf; m.ng = nc - nci;
  m.ldc = pad32(nc); m.ldf = pad32(nf);
  const size_t lf = m.ldf, lc = m.ldc;
  // ---- connectivity ----
  h->fc1.resize(nf); h->fc2.resize(nf);
  std::vector<int> fbc(nf), part(nf, -1);
  for (int f = 0; f < nf; ++f) {
    int a = d->facecell[f] - 1, b = d->facecell[nf + f] - 1;
    if (a < 0 || a >= nci || b < 0 || b >= nc) { tyi::set_error("facecell out of range at face " + std::to_string(f)); return bail(TY_ERR_MESH); }
    h->fc1[f] = a; h->fc2[f] = b;
    fbc[f] = f < nfi ? TY_BC_INTERIOR : d->face_bc[f];
    if (f < nfi && b >= nci) { tyi::set_error("interior face with a ghost cell"); return bail(TY_ERR_MESH); }
    if (f >= nfi) {
      if (b < nci) { tyi::set_error("boundary face without ghost cell"); return bail(TY_ERR_MESH); }
      if (fbc[f] != TY_BC_PERIODIC) h->nonperiodic_bc = true;
      if (fbc[f] == TY_BC_PERIODIC) {
        int p = d->face_partner[f] - 1;
        if (p < nfi || p >= nf || d->face_partner[p] - 1 != f) { tyi::set_error("bad periodic partner"); return bail(TY_ERR_MESH); }
        part[f] = p;
      } else if (fbc[f] == TY_BC_HEAT) {
        h->heat_bc = true;
      } else if (fbc[f] >= TY_BC_INLET_SUB && fbc[f] <= TY_BC_OUTLET_SUP) {
        h->inout_bc = true;
      } else if (fbc[f] != TY_BC_SYMMETRY && fbc[f] != TY_BC_WALL && fbc[f] != TY_BC_FARFIELD &&
                 fbc[f] != TY_BC_NOSLIP) {
        tyi::set_error("unknown boundary kind");
        return bail(TY_ERR_UNSUPPORTED);
      }
    }
  }
  // ghosts
  const int ng = m.ng;
  std::vector<int> gsrc(std::max(ng, 1), -1), gface(std::max(ng, 1), -1);
  for (int f = nfi; f < nf; ++f) {
    int k = h->fc2[f] - nci;
    if (gface[k] >= 0) { tyi::set_error("ghost cell shared by two faces"); return bail(TY_ERR_MESH); }
    gface[k] = f;
    gsrc[k] = part[f] >= 0 ? h->fc1[part[f]] : h->fc1[f];
  }
  // wall ghosts: |F - C|^2 / |(F - C).n|  (setboco_ns_flux.f90, cell-state mode)
  std::vector<double> gdist(std::max(ng, 1), 0.0);
  for (int k = 0; k < ng; ++k) {
    const int f = gface[k];
    if (fbc[f] != TY_BC_WALL && fbc[f] != TY_BC_NOSLIP) continue;
    const double* F = &d->face_centre[3 * (size_t)f];
    const double* Cc = &d->cell_centre[3 * (size_t)h->fc1[f]];
    const double* n = &d->face_normal[3 * (size_t)f];
    const double a0 = F[0] - Cc[0], a1 = F[1] - Cc[1], a2 = F[2] - Cc[2];
    gdist[k] = (a0 * a0 + a1 * a1 + a2 * a2) / std::fabs(a0 * n[0] + a1 * n[1] + a2 * n[2]);
  }
  // gather lists in colour order
  std::vector<std::vector<std::pair<int, int>>> lists(nci);
  for (int f = 0; f < nf; ++f) {
    lists[h->fc1[f]].push_back({d->face_color[f], f << 1});
    if (h->fc2[f] < nci) lists[h->fc2[f]].push_back({d->face_color[f], (f << 1) | 1});
  }
  int nslot = 0;
  for (auto& l : lists) {
    std::sort(l.begin(), l.end());
    for (size_t i = 1; i < l.size(); ++i)
      if (l[i].first == l[i - 1].first) { tyi::set_error("two faces of one cell share a colour"); return bail(TY_ERR_MESH); }
    nslot = std::max(nslot, (int)l.size());
  }
  if (nslot > kMaxSlot) { tyi::set_error("more than 8 faces per cell"); return bail(TY_ERR_UNSUPPORTED); }
  m.nslot = nslot;
  h->cf.assign((size_t)nslot * nci, -1);
  std::vector<int> cfn((size_t)nslot * nci, -1);
  std::vector<double> sumS(nci, 0.0);
  for (int c = 0; c < nci; ++c)
    for (size_t i = 0; i < lists[c].size(); ++i) {
      int e = lists[c][i].second;
      int f = e >> 1;
      h->cf[i * (size_t)nci + c] = e;
      cfn[i * (size_t)nci + c] = (e & 1) ? h->fc1[f] : h->fc2[f];
      sumS[c] = sumS[c] + d->face_surface[f];
    }
  std::vector<double> invV(nci), geo2(nci);
  for (int c = 0; c < nci; ++c) {
    if (!(d->cell_volume[c] > 0.0) || !(sumS[c] > 0.0)) { tyi::set_error("non-positive cell volume or surface"); return bail(TY_ERR_MESH); }
    invV[c] = 1.0 / d->cell_volume[c];
    geo2[c] = 2.0 * d->cell_volume[c] / sumS[c];
  }
  // geometry
  h->ccentre.assign(d->cell_centre, d->cell_centre + 3 * (size_t)nc);
  h->fcentre.assign(d->face_centre, d->face_centre + 3 * (size_t)nf);
  h->fnormal.assign(d->face_normal, d->face_normal + 3 * (size_t)nf);
  h->cvol.assign(d->cell_volume, d->cell_volume + (size_t)nc);
  h->fsurf.assign(d->face_surface, d->face_surface + (size_t)nf);
  std::vector<double> fn(3 * lf, 0.0), fs(lf, 0.0), fw(3 * lf, 0.0), cv(lc, 0.0);
  for (int f = 0; f < nf; ++f) {
    for (int k = 0; k < 3; ++k) {
      fn[k * lf + f] = d->face_normal[3 * (size_t)f + k];
      if (d->face_wallvel) fw[k * lf + f] = d->face_wallvel[3 * (size_t)f + k];
    }
    fs[f] = d->face_surface[f];
  }
  for (int c = 0; c < nc; ++c) cv[c] = d->cell_volume[c];
  int rc;
  if ((rc = h->upload(m.fc1, h->fc1)) || (rc = h->upload(m.fc2, h->fc2)) || (rc = h->upload(m.fbc, fbc)) ||
      (rc = h->upload(m.part, part)) || (rc = h->upload(m.cf, h->cf)) || (rc = h->upload(m.gsrc, gsrc)) ||
      (rc = h->upload(m.gface, gface)) || (rc = h->upload(m.fn, fn)) || (rc = h->upload(m.fs, fs)) ||
      (rc = h->upload(m.fwall, fw)) || (rc = h->upload(m.cvol, cv)) || (rc = h->upload(m.sumS, sumS)) ||
      (rc = h->upload(m.cfn, cfn)) || (rc = h->upload(m.invV, invV)) || (rc = h->upload(m.geo2, geo2)) ||
      (rc = h->upload(m.gdist, gdist)))
    return bail(rc);
  // state
  DevState& s = h->s;
  if ((rc = h->alloc(s.u0, 5 * lc)) || (rc = h->alloc(s.cur, 5 * lc)) || (rc = h->alloc(s.acc, 5 * lc)) ||
      (rc = h->alloc(s.prim, 5 * lc)) || (rc = h->alloc(s.grad, 15 * lc)) || (rc = h->alloc(s.ratio, 3 * lc)) ||
      (rc = h->alloc(s.flux, 5 * lf)) || (rc = h->alloc(s.res, 5 * lc)) || (rc = h->alloc(s.dtbits, 4)) ||
      (rc = h->alloc(s.stage, 5 * (size_t)nci)) ||
      (rc = h->alloc(s.err, 4)))
    return bail(rc);
  TY_CU(cudaMemset(s.u0, 0, 5 * lc * sizeof(double)));
  TY_CU(cudaMemset(s.grad, 0, 15 * lc * sizeof(double)));
  TY_CU(cudaMemset(s.prim, 0, 5 * lc * sizeof(double)));
  TY_CU(cudaMemset(s.err, 0, 4 * sizeof(int)));
  TY_CU(cudaMemset(s.ratio, 0, 3 * lc * sizeof(double)));
  if (cudaMallocHost((void**)&h->dtbits_host, 4 * sizeof(double)) != cudaSuccess) return bail(TY_ERR_NOMEM);
  h->nslot = nslot;
  *out = h;
  return TY_OK;
}

int ty_mesh_destroy(ty_mesh* h) {
  if (!h) return TY_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* p : h->allocs) cudaFree(p);
  if (h->dtbits_host) cudaFreeHost(h->dtbits_host);
  if (h->imp.pinned) cudaFreeHost(h->imp.pinned);
  if (h->kd.pinned) cudaFreeHost(h->kd.pinned);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return TY_OK;
}

int ty_mesh_info(const ty_mesh* h, int32_t* out) {
  if (!h || !out) return TY_ERR_ARG;
  out[0] = h->m.nci; out[1] = h->m.nc; out[2] = h->m.nfi; out[3] = h->m.nf; out[4] = h->m.nslot;
  return TY_OK;
}

int ty_set_bc_data(ty_mesh* h, const double* data) {
  if (!h || !data) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  const int nf = h->m.nf;
  const size_t lf = h->m.ldf;
  std::vector<double> d(6 * lf, 0.0);
  for (int f = 0; f < nf; ++f)
    for (int q = 0; q < 6; ++q) d[q * lf + f] = data[6 * (size_t)f + q];
  if (!h->m.fbcd) {
    if (int rc = h->upload(h->m.fbcd, d)) return rc;
  } else {
    TY_CU(cudaMemcpy(const_cast<double*>(h->m.fbcd), d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  h->bcdata_set = true;
  h->prim_valid = false;
  return TY_OK;
}

int ty_mesh_set_face_rotation(ty_mesh* h, const double* rot) {
  if (!h || !rot) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  const int nf = h->m.nf;
  const size_t lf = h->m.ldf;
  std::vector<double> d(9 * lf, 0.0);
  bool any = false;
  for (int f = 0; f < nf; ++f)
    for (int q = 0; q < 9; ++q) {
      const double v = rot[9 * (size_t)f + q];
      d[q * lf + f] = v;
      any = any || v != ((q % 4 == 0) ? 1.0 : 0.0);
    }
  if (!any) return TY_OK;  // translations only: nothing to rotate
  if (!h->m.frot) {
    if (int rc = h->upload(h->m.frot, d)) return rc;
  } else {
    TY_CU(cudaMemcpy(const_cast<double*>(h->m.frot), d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  h->prim_valid = false;
  return TY_OK;
}

int ty_set_params(ty_mesh* h, const ty_spat_params* p) {
  if (!h || !p) return TY_ERR_ARG;
  if (p->scheme < TY_SCH_HLLC || p->scheme > TY_SCH_HLLEKB || p->highres < 0 || p->highres > TY_HRES_MUSCLUNS ||
      p->limiter < 0 || p->limiter > TY_LIM_LIM03 || p->postlim < 0 || p->postlim > TY_POSTLIM_SUPERBARTH ||
      p->gradmeth < 0 || p->gradmeth > TY_GRAD_LSQW || (p->mode != TY_MODE_EXACT && p->mode != TY_MODE_FAST) ||
      !(p->gamma > 1.0)) {
    tyi::set_error("ty_spat_params: value out of range");
    return TY_ERR_ARG;
  }
  if (p->highres != TY_HRES_NONE && p->gradmeth == TY_GRAD_NONE) {
    tyi::set_error("MUSCL reconstruction needs a gradient method");
    return TY_ERR_ARG;
  }
  if (p->viscous < TY_VISC_NONE || p->viscous > TY_VISC_CELLFULL || p->visc_law < TY_VISC_KINEMATIC ||
      p->visc_law > TY_VISC_SUTHERLAND) {
    tyi::set_error("ty_spat_params: viscous option out of range");
    return TY_ERR_ARG;
  }
  if (p->viscous != TY_VISC_NONE &&
      (p->gradmeth == TY_GRAD_NONE || !(p->rgas > 0.0) || !(p->prandtl > 0.0) ||
       (p->visc_law == TY_VISC_KINEMATIC && !(p->visc_kin >= 0.0)))) {
    tyi::set_error("the viscous flux needs cell gradients, rgas > 0, prandtl > 0 and a viscosity");
    return TY_ERR_ARG;
  }
  TY_CU(cudaSetDevice(h->device));
  int rc;
  if (p->gradmeth != TY_GRAD_NONE && h->lsq_gradmeth != p->gradmeth)
    if ((rc = build_lsq(h, p->gradmeth))) return rc;
  if (p->highres != TY_HRES_NONE && h->geo_highres != p->highres)
    if ((rc = build_muscl_geometry(h, p->highres))) return rc;
  if (p->viscous != TY_VISC_NONE && !h->visc_ready)
    if ((rc = build_viscous_geometry(h))) return rc;
  if ((p->postlim != TY_POSTLIM_NONE || (p->mode == TY_MODE_FAST && p->highres != TY_HRES_NONE)) && !h->s.cl) {
    if ((rc = h->alloc(h->s.cl, 5 * (size_t)h->m.ldf)) || (rc = h->alloc(h->s.cr, 5 * (size_t)h->m.ldf))) return rc;
  }
  // fast MUSCL / MUSCL-UNS without limiter: the per-cell increment matrices of k_cell_fast
  h->m.mtab = nullptr;
  if (p->mode == TY_MODE_FAST && (p->highres == TY_HRES_MUSCL || p->highres == TY_HRES_MUSCLUNS) &&
      p->limiter == TY_LIM_NONE && p->gradmeth != TY_GRAD_NONE && h->m.nslot > 0) {
    if (!h->mtab_buf && (rc = h->alloc(h->mtab_buf, (size_t)h->m.nslot * h->m.nslot * (size_t)h->m.nci))) return rc;
    cudaError_t e = tyk::kfast::build_mtab(h->m, h->mtab_buf, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "increment matrices");
    h->m.mtab = h->mtab_buf;
  }
  h->o.scheme = p->scheme; h->o.highres = p->highres; h->o.limiter = p->limiter; h->o.postlim = p->postlim;
  h->o.gradmeth = p->gradmeth; h->o.mode = p->mode; h->o.gamma = p->gamma; h->o.entropy_fix = p->entropy_fix;
  h->o.inv_entropy_fix = p->entropy_fix > 0.0 ? 1.0 / p->entropy_fix : 0.0;
  h->o.ig1 = 1.0 / (p->gamma - 1.0);
  h->o.gig1 = p->gamma * h->o.ig1;
  {  // the HLL family's wave-speed variant (def_spat.f90:68-76, calc_flux_hllc.f90:64-72)
    const int sc = p->scheme;
    h->o.hll_family = (sc == TY_SCH_HLLC || (sc >= TY_SCH_HLLCB && sc <= TY_SCH_HLLCKB)) ? 1
                      : (sc == TY_SCH_HLLE || (sc >= TY_SCH_HLLEB && sc <= TY_SCH_HLLEKB)) ? 2 : 0;
    const bool b = sc == TY_SCH_HLLCB || sc == TY_SCH_HLLCKB || sc == TY_SCH_HLLEB || sc == TY_SCH_HLLEKB;
    h->o.hll_kin = (sc == TY_SCH_HLLCK || sc == TY_SCH_HLLCKB || sc == TY_SCH_HLLEK || sc == TY_SCH_HLLEKB) ? 1 : 0;
    h->o.hll_beta = b ? std::sqrt((p->gamma - 1.0) / (2 * p->gamma)) : 1.0;
    h->o.hll_f1 = std::sqrt(0.5 * p->gamma);
    h->o.hll_f2 = 0.5 / std::sqrt(3.141592653589793238462643);
  }
  h->o.viscous = p->viscous; h->o.visc_law = p->visc_law; h->o.visc_kin = p->visc_kin;
  h->o.rgas = p->rgas; h->o.prandtl = p->prandtl;
  for (int v = 0; v < 5; ++v) h->o.farfield[v] = p->farfield[v];
  h->has_params = true;
  h->prim_valid = false;
  return TY_OK;
}

int ty_state_upload(ty_mesh* h, const double* rho, const double* rhoE, const double* rhou) {
  if (!h || !rho || !rhoE || !rhou) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  const size_t n = h->m.nci;
  // copy Typhon's layout as is (pinned caller buffers go straight over DMA), transpose on the GPU
  TY_CU(cudaMemcpyAsync(h->s.stage, rho, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TY_CU(cudaMemcpyAsync(h->s.stage + n, rhoE, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TY_CU(cudaMemcpyAsync(h->s.stage + 2 * n, rhou, 3 * n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  cudaError_t e = tyk::kexact::unpack_state(h->m, h->s, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "unpack state");
  TY_CU(cudaStreamSynchronize(h->stream));
  h->has_state = true;
  h->prim_valid = false;
  return TY_OK;
}

int ty_state_download(ty_mesh* h, double* rho, double* rhoE, double* rhou) {
  if (!h || !rho || !rhoE || !rhou) return TY_ERR_ARG;
  if (!h->has_state) return TY_ERR_STATE;
  TY_CU(cudaSetDevice(h->device));
  const size_t n = h->m.nci;
  cudaError_t e = tyk::kexact::pack_state(h->m, h->s, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "pack state");
  TY_CU(cudaMemcpyAsync(rho, h->s.stage, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TY_CU(cudaMemcpyAsync(rhoE, h->s.stage + n, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TY_CU(cudaMemcpyAsync(rhou, h->s.stage + 2 * n, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

int ty_state_upload_device(ty_mesh* h, const double* cons) {
  if (!h || !cons) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  const int n = h->m.nci;
  TY_CU(cudaMemcpy2DAsync(h->s.u0, h->m.ldc * sizeof(double), cons, n * sizeof(double), n * sizeof(double), 5,
                          cudaMemcpyDeviceToDevice, h->stream));
  h->has_state = true;
  h->prim_valid = false;
  return TY_OK;
}

int ty_state_download_device(ty_mesh* h, double* cons) {
  if (!h || !cons) return TY_ERR_ARG;
  if (!h->has_state) return TY_ERR_STATE;
  TY_CU(cudaSetDevice(h->device));
  const int n = h->m.nci;
  TY_CU(cudaMemcpy2DAsync(cons, n * sizeof(double), h->s.u0, h->m.ldc * sizeof(double), n * sizeof(double), 5,
                          cudaMemcpyDeviceToDevice, h->stream));
  return TY_OK;
}

int ty_prim_download(ty_mesh* h, double* prim) {
  int rc = ready(h);
  if (rc) return rc;
  if ((rc = ensure_prim(h))) return rc;
  const int n = h->m.nci;
  TY_CU(cudaMemcpy2DAsync(prim, n * sizeof(double), h->s.prim, h->m.ldc * sizeof(double), n * sizeof(double), 5,
                          cudaMemcpyDeviceToHost, h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

int ty_timestep(ty_mesh* h, double cfl, double* dt_out) {
  int rc = ready(h);
  if (rc) return rc;
  if (!dt_out || !(cfl > 0.0)) return TY_ERR_ARG;
  if ((rc = set_dt_slot(h, 2, 1.7976931348623157e308))) return rc;
  cudaError_t e = MODE_CALL(h, timestep, h->m, h->s, h->o, h->s.u0, cfl, h->s.dtbits + 2, h->stream, &h->prof);
  if (e != cudaSuccess) return cuda_fail(e, "timestep");
  unsigned long long b = 0;
  TY_CU(cudaMemcpyAsync(&b, h->s.dtbits + 2, 8, cudaMemcpyDeviceToHost, h->stream));
  if ((rc = check_err(h))) return rc;
  double dt;
  std::memcpy(&dt, &b, 8);
  if (dt != dt) return TY_ERR_NANDT;
  *dt_out = dt;
  return TY_OK;
}

int ty_residual(ty_mesh* h, double dt, double* R_out) {
  int rc = ready(h);
  if (rc) return rc;
  if ((rc = ensure_prim(h))) return rc;
  if ((rc = stage_faces(h))) return rc;
  cudaError_t e = MODE_CALL(h, residual_gather, h->m, h->s, dt, nullptr, h->stream, &h->prof);
  if (e != cudaSuccess) return cuda_fail(e, "residual gather");
  if (R_out) {
    const int n = h->m.nci;
    TY_CU(cudaMemcpy2DAsync(R_out, n * sizeof(double), h->s.res, h->m.ldc * sizeof(double), n * sizeof(double), 5,
                            cudaMemcpyDeviceToHost, h->stream));
  }
  TY_CU(cudaStreamSynchronize(h->stream));
  return check_err(h);
}

int ty_rk_step(ty_mesh* h, int32_t method, double dt) {
  int rc = ready(h);
  if (rc) return rc;
  RkTab t;
  if (!rk_table(method, t) || !(dt >= 0.0)) return TY_ERR_ARG;
  if ((rc = run_step(h, t, dt, nullptr, nullptr, 0.0))) return rc;
  TY_CU(cudaStreamSynchronize(h->stream));
  return check_err(h);
}

int ty_rk_steps(ty_mesh* h, int32_t method, double cfl, int32_t nsteps, double* dt_last) {
  int rc = ready(h);
  if (rc) return rc;
  RkTab t;
  if (!rk_table(method, t) || nsteps < 0 || !(cfl > 0.0)) return TY_ERR_ARG;
  if (nsteps == 0) return TY_OK;
  // slot 0/1 alternate: step n reads slot n%2, its last stage writes the next dt into the other
  if ((rc = set_dt_slot(h, 0, 1.7976931348623157e308))) return rc;
  cudaError_t e = MODE_CALL(h, timestep, h->m, h->s, h->o, h->s.u0, cfl, h->s.dtbits, h->stream, &h->prof);
  if (e != cudaSuccess) return cuda_fail(e, "timestep");
  for (int n = 0; n < nsteps; ++n) {
    int cur = n & 1, nxt = cur ^ 1;
    if ((rc = set_dt_slot(h, nxt, 1.7976931348623157e308))) return rc;
    if ((rc = run_step(h, t, 0.0, h->s.dtbits + cur, h->s.dtbits + nxt, cfl))) return rc;
  }
  if (dt_last) {
    unsigned long long b;
    TY_CU(cudaMemcpyAsync(&b, h->s.dtbits + ((nsteps - 1) & 1), 8, cudaMemcpyDeviceToHost, h->stream));
    TY_CU(cudaStreamSynchronize(h->stream));
    std::memcpy(dt_last, &b, 8);
  }
  TY_CU(cudaStreamSynchronize(h->stream));
  return check_err(h);
}

int ty_steady_iteration(ty_mesh* h, int32_t method, double cfl, int32_t local_dt, double* dt_out, double* res_l1) {
  int rc = ready(h);
  if (rc) return rc;
  RkTab t;
  if (!rk_table(method, t) || !(cfl > 0.0) || !res_l1) return TY_ERR_ARG;
  if (!h->steady_red && (rc = h->alloc(h->steady_red, 3 * (size_t)tyk::kRedBlocks + 3))) return rc;
  if (local_dt && !h->steady_dtloc && (rc = h->alloc(h->steady_dtloc, (size_t)h->m.nci))) return rc;
  if ((rc = set_dt_slot(h, 0, 1.7976931348623157e308))) return rc;
  cudaError_t e;
  if (local_dt) {  // calc_ns_timestep per cell, kept per cell (calc_zonetimestep.f90:93-117, loc_stab_cond)
    tyk::ImpState im = h->imp;
    im.dtloc = h->steady_dtloc;
    e = MODE_CALL(h, imp_dtloc, h->m, h->s, h->o, im, cfl, h->s.dtbits, h->stream);
  } else {
    e = MODE_CALL(h, timestep, h->m, h->s, h->o, h->s.u0, cfl, h->s.dtbits, h->stream, &h->prof);
  }
  if (e != cudaSuccess) return cuda_fail(e, "timestep");
  if ((rc = run_step(h, t, 0.0, h->s.dtbits, nullptr, cfl, true, local_dt ? h->steady_dtloc : nullptr))) return rc;
  double* out = h->steady_red + 3 * (size_t)tyk::kRedBlocks;
  e = MODE_CALL(h, res_l1, h->m.nci, h->s.acc, (size_t)h->m.ldc, h->steady_red, out, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "residual sums");
  TY_CU(cudaMemcpyAsync(res_l1, out, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (dt_out) {
    unsigned long long b;
    TY_CU(cudaMemcpyAsync(&b, h->s.dtbits, 8, cudaMemcpyDeviceToHost, h->stream));
    TY_CU(cudaStreamSynchronize(h->stream));
    std::memcpy(dt_out, &b, 8);
  }
  TY_CU(cudaStreamSynchronize(h->stream));
  return check_err(h);
}

int ty_ghost_state_set(ty_mesh* h, const double* cons_ghost) {
  if (!h) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  if (!cons_ghost) {
    h->ghost_rows = false;
    return TY_OK;
  }
  const size_t ng = (size_t)h->m.ng;
  if (ng == 0) {
    tyi::set_error("ty_ghost_state_set: the mesh has no ghost cells");
    return TY_ERR_ARG;
  }
  int rc;
  if (!h->gcons && ((rc = h->alloc(h->gcons, 5 * ng)) || (rc = h->alloc(h->gres, (size_t)kMaxStage * 5 * ng)) ||
                    (rc = h->alloc(h->gprim, 5 * ng))))
    return rc;
  TY_CU(cudaMemcpyAsync(h->gcons, cons_ghost, 5 * ng * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TY_CU(cudaMemsetAsync(h->gprim, 0, 5 * ng * sizeof(double), h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  h->ghost_rows = true;
  return TY_OK;
}

int ty_ghost_prim_download(ty_mesh* h, double* prim_ghost) {
  if (!h || !prim_ghost) return TY_ERR_ARG;
  if (!h->ghost_rows) {
    tyi::set_error("ty_ghost_prim_download: no ghost state (ty_ghost_state_set)");
    return TY_ERR_STATE;
  }
  TY_CU(cudaSetDevice(h->device));
  TY_CU(cudaMemcpyAsync(prim_ghost, h->gprim, 5 * (size_t)h->m.ng * sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

int ty_debug_get(ty_mesh* h, int32_t which, double* out) {
  if (!h || !out) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  const DevMesh& m = h->m;
  const double* src;
  int rows, n;
  size_t ld;
  switch (which) {
    case 0: src = h->s.prim; rows = 5; n = m.nc; ld = m.ldc; break;
    case 1: src = h->s.grad; rows = 15; n = m.nc; ld = m.ldc; break;
    case 2: src = h->s.flux; rows = 5; n = m.nf; ld = m.ldf; break;
    case 3: src = h->s.ratio; rows = 3; n = m.nc; ld = m.ldc; break;
    default: return TY_ERR_ARG;
  }
  TY_CU(cudaMemcpy2DAsync(out, n * sizeof(double), src, ld * sizeof(double), n * sizeof(double), rows,
                          cudaMemcpyDeviceToHost, h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

int ty_set_stream(ty_mesh* h, void* stream) {
  if (!h) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  TY_CU(cudaStreamSynchronize(h->stream));
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return TY_OK;
}

int ty_profile_enable(ty_mesh* h, int32_t on) {
  if (!h) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  TY_CU(cudaStreamSynchronize(h->stream));
  h->prof.reset();
  h->prof.on = on != 0;
  return TY_OK;
}

int ty_profile_read(ty_mesh* h, int32_t n, double* ms, int32_t* launches) {
  if (!h || !ms || !launches || n < 0) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  TY_CU(cudaStreamSynchronize(h->stream));
  for (int i = 0; i < n; ++i) { ms[i] = 0.0; launches[i] = 0; }
  for (auto& r : h->prof.rec) {
    float t = 0.f;
    TY_CU(cudaEventElapsedTime(&t, r.a, r.b));
    if (r.id < n) { ms[r.id] += t; launches[r.id] += 1; }
  }
  return TY_OK;
}

int ty_synchronize(ty_mesh* h) {
  if (!h) return TY_ERR_ARG;
  TY_CU(cudaSetDevice(h->device));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

}  // extern "C"
