// Heat conduction (KDIF) of libtyphon_gpu: set-up, residual, implicit step, accessors.
//
// The face geometry of calc_kdif_flux.f90:76-96 (normalised distances HL, HR, C_R - C_L,
// (d.n), |d|^2) is computed once on the host in the oracle's operation order.  The implicit
// step assembles the symmetrised system diag(V/dt) A (symmetric positive definite: A is
// Typhon's DLU matrix I + dt/V J with the compact Jacobian J_R = -k (d.n) / (Cp |d|^2),
// J_L = -J_R) and solves it by Jacobi-preconditioned conjugate gradients in FP64 (one fused
// pair of launches per iteration, kdif.cuh), by the same iteration on FP32 conductances until
// 1e-6 and then on FP64 ones (mixed), or by FP32 conjugate gradients inside FP64 iterative
// refinement.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "handle.hpp"

using namespace tyk;
using namespace tyi;

#define KD_CALL(h, fn, ...) \
  ((h)->o.mode == TY_MODE_FAST ? tyk::kfast::fn(__VA_ARGS__) : tyk::kexact::fn(__VA_ARGS__))

namespace {

int fetch(ty_mesh* h, int off, int k) {
  TY_CU(cudaMemcpyAsync(h->kd.pinned + off, h->kd.scal + off, k * sizeof(double), cudaMemcpyDeviceToHost,
                        h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

int kd_ready(ty_mesh* h) {
  if (!h) return TY_ERR_ARG;
  if (!h->kd.ready) { tyi::set_error("call ty_kdif_setup first"); return TY_ERR_STATE; }
  TY_CU(cudaSetDevice(h->device));
  return TY_OK;
}

}  // namespace

extern "C" {

int ty_kdif_setup(ty_mesh* h, const ty_kdif_params* p, const double* conductivity, const int32_t* face_kind,
                  const double* face_value) {
  if (!h || !p || !conductivity || !face_kind || !face_value) return TY_ERR_ARG;
  if (p->flux < TY_KDIF_COMPACT || p->flux > TY_KDIF_FULL || !(p->heat_capacity > 0.0)) {
    tyi::set_error("ty_kdif_params: flux scheme or heat capacity out of range");
    return TY_ERR_ARG;
  }
  TY_CU(cudaSetDevice(h->device));
  if (h->m.frot) {
    tyi::set_error("ty_kdif_setup: heat conduction on meshes with rotational periodicity is not built");
    return TY_ERR_UNSUPPORTED;
  }
  DevMesh& m = h->m;
  KdifState& k = h->kd;
  const int nci = m.nci, nc = m.nc, nf = m.nf, nfi = m.nfi;
  std::vector<int> kind(nf, 0);
  std::vector<double> kc(m.ldc, 0.0), val(nf, 0.0);
  for (int c = 0; c < nci; ++c) {
    if (!(conductivity[c] > 0.0)) { tyi::set_error("non-positive conductivity at cell " + std::to_string(c)); return TY_ERR_ARG; }
    kc[c] = conductivity[c];
  }
  std::vector<int> gsrc(nc - nci);
  TY_CU(cudaMemcpy(gsrc.data(), m.gsrc, gsrc.size() * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> fbc(nf);
  TY_CU(cudaMemcpy(fbc.data(), m.fbc, nf * sizeof(int), cudaMemcpyDeviceToHost));
  for (int f = nfi; f < nf; ++f) {
    if (fbc[f] != TY_BC_PERIODIC) {
      if (face_kind[f] < TY_KBC_ISOTHERMAL || face_kind[f] > TY_KBC_EXTRAPOLATE) {
        tyi::set_error("boundary face " + std::to_string(f) + " without a ty_kdif_bc kind");
        return TY_ERR_ARG;
      }
      kind[f] = face_kind[f];
      val[f] = face_value[f];
    }
  }
  for (int g = 0; g < nc - nci; ++g) kc[nci + g] = kc[gsrc[g]];
  h->kd_k.assign(kc.begin(), kc.begin() + nci);
  // calc_kdif_flux.f90:83-91 geometry, in the oracle's operation order
  const size_t lf = m.ldf;
  std::vector<double> geo(7 * lf, 0.0);
  for (int f = 0; f < nf; ++f) {
    const double* CL = &h->ccentre[3 * (size_t)h->fc1[f]];
    const double* CR = &h->ccentre[3 * (size_t)h->fc2[f]];
    const double* F = &h->fcentre[3 * (size_t)f];
    const double a0 = F[0] - CL[0], a1 = F[1] - CL[1], a2 = F[2] - CL[2];
    const double b0 = F[0] - CR[0], b1 = F[1] - CR[1], b2 = F[2] - CR[2];
    double dHL = std::sqrt(a0 * a0 + a1 * a1 + a2 * a2), dHR = std::sqrt(b0 * b0 + b1 * b1 + b2 * b2);
    const double id = 1.0 / (dHL + dHR);
    dHL = id * dHL;
    dHR = id * dHR;
    const double v0 = CR[0] - CL[0], v1 = CR[1] - CL[1], v2 = CR[2] - CL[2];
    const double dLR = std::sqrt(v0 * v0 + v1 * v1 + v2 * v2);
    const double* n = &h->fnormal[3 * (size_t)f];
    geo[f] = dHL; geo[lf + f] = dHR;
    geo[2 * lf + f] = v0; geo[3 * lf + f] = v1; geo[4 * lf + f] = v2;
    geo[5 * lf + f] = v0 * n[0] + v1 * n[1] + v2 * n[2];
    geo[6 * lf + f] = dLR * dLR;
  }
  int rc;
  if (!k.T) {
    // face lists in ascending face order
    const int ns = m.nslot;
    std::vector<std::vector<int>> l(nci);
    for (int f = 0; f < nf; ++f) {
      l[h->fc1[f]].push_back(f << 1);
      if (h->fc2[f] < nci) l[h->fc2[f]].push_back((f << 1) | 1);
    }
    std::vector<int> cfo((size_t)ns * nci, -1), cfon((size_t)ns * nci, -1);
    for (int c = 0; c < nci; ++c) {
      std::sort(l[c].begin(), l[c].end());
      for (size_t i = 0; i < l[c].size(); ++i) {
        const int e = l[c][i], f = e >> 1;
        cfo[i * (size_t)nci + c] = e;
        cfon[i * (size_t)nci + c] = (e & 1) ? h->fc1[f] : h->fc2[f];
      }
    }
    if ((rc = h->alloc(k.k, (size_t)m.ldc)) || (rc = h->alloc(k.fkind, (size_t)nf)) ||
        (rc = h->alloc(k.fval, (size_t)nf)) || (rc = h->alloc(k.T, (size_t)m.ldc)) ||
        (rc = h->alloc(k.grad, 3 * (size_t)m.ldc)) || (rc = h->alloc(k.flux, (size_t)nf)) ||
        (rc = h->alloc(k.jac, (size_t)nf)) || (rc = h->alloc(k.diag, (size_t)nci)) ||
        (rc = h->alloc(k.bal, (size_t)nci)) || (rc = h->alloc(k.x, (size_t)nci)) || (rc = h->alloc(k.r, (size_t)nci)) ||
        (rc = h->alloc(k.z, (size_t)nci)) || (rc = h->alloc(k.p, (size_t)nci)) || (rc = h->alloc(k.q, (size_t)nci)) ||
        (rc = h->alloc(k.r32, (size_t)nci)) || (rc = h->alloc(k.z32, (size_t)nci)) ||
        (rc = h->alloc(k.p32, (size_t)nci)) || (rc = h->alloc(k.q32, (size_t)nci)) ||
        (rc = h->alloc(k.x32, (size_t)nci)) || (rc = h->alloc(k.diag32, (size_t)nci)) ||
        (rc = h->alloc(k.jac32, (size_t)nf)) || (rc = h->alloc(k.part, 4 * (size_t)kRedBlocks)) ||
        (rc = h->alloc(k.scal, (size_t)16)) || (rc = h->alloc(k.cfo, cfo.size())) || (rc = h->alloc(k.cfon, cfon.size())) ||
        (rc = h->alloc(k.ell_m, (size_t)nci)) || (rc = h->alloc(k.ell_a, (size_t)ns * nci)) ||
        (rc = h->alloc(k.ell_a32, (size_t)ns * nci)) || (rc = h->alloc(k.ell_nb, (size_t)ns * nci)) ||
        (rc = h->alloc(k.dinv, (size_t)nci)) || (rc = h->alloc(k.s, (size_t)nci)) || (rc = h->alloc(k.count, 2)))
      return rc;
    TY_CU(cudaMemset(k.count, 0, 2 * sizeof(unsigned)));
    TY_CU(cudaMemcpy(k.cfo, cfo.data(), cfo.size() * sizeof(int), cudaMemcpyHostToDevice));
    TY_CU(cudaMemcpy(k.cfon, cfon.data(), cfon.size() * sizeof(int), cudaMemcpyHostToDevice));
    TY_CU(cudaMemset(k.T, 0, m.ldc * sizeof(double)));
    TY_CU(cudaMemset(k.grad, 0, 3 * m.ldc * sizeof(double)));
    if (cudaMallocHost((void**)&k.pinned, 16 * sizeof(double)) != cudaSuccess) return TY_ERR_NOMEM;
  }
  if ((rc = h->upload(k.kgeo, geo))) return rc;
  TY_CU(cudaMemcpy(k.k, kc.data(), m.ldc * sizeof(double), cudaMemcpyHostToDevice));
  TY_CU(cudaMemcpy(k.fkind, kind.data(), nf * sizeof(int), cudaMemcpyHostToDevice));
  TY_CU(cudaMemcpy(k.fval, val.data(), nf * sizeof(double), cudaMemcpyHostToDevice));
  if (p->flux != TY_KDIF_COMPACT && (rc = ensure_lsq(h))) return rc;
  k.scheme = p->flux;
  k.cp = p->heat_capacity;
  k.ready = true;
  return TY_OK;
}

int ty_kdif_set_temperature(ty_mesh* h, const double* T) {
  if (int rc = kd_ready(h)) return rc;
  if (!T) return TY_ERR_ARG;
  TY_CU(cudaMemcpyAsync(h->kd.T, T, h->m.nci * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

int ty_kdif_get_temperature(ty_mesh* h, double* T) {
  if (int rc = kd_ready(h)) return rc;
  if (!T) return TY_ERR_ARG;
  TY_CU(cudaMemcpyAsync(T, h->kd.T, h->m.nci * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

int ty_kdif_residual(ty_mesh* h, double dt, double* R) {
  if (int rc = kd_ready(h)) return rc;
  TY_CU(KD_CALL(h, kdif_residual, h->m, h->kd, dt, h->stream));
  if (R) {
    std::vector<double> bal(h->m.nci);
    TY_CU(cudaMemcpyAsync(bal.data(), h->kd.bal, bal.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TY_CU(cudaStreamSynchronize(h->stream));
    for (int c = 0; c < h->m.nci; ++c) R[c] = dt / h->cvol[c] * bal[c];
  }
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

int ty_kdif_implicit_step(ty_mesh* h, double dt, const ty_kdif_solve* s, ty_kdif_stats* st) {
  if (int rc = kd_ready(h)) return rc;
  if (!s || !st || !(dt > 0.0) || !(s->tol > 0.0) || s->max_it < 1 ||
      (s->solver != TY_KSOLVE_CG && s->solver != TY_KSOLVE_CG32_REFINE && s->solver != TY_KSOLVE_CG_MIXED)) {
    tyi::set_error("ty_kdif_implicit_step: bad dt or solver parameters");
    return TY_ERR_ARG;
  }
  std::memset(st, 0, sizeof(*st));
  const DevMesh& m = h->m;
  KdifState& k = h->kd;
  cudaStream_t q = h->stream;
  const bool f32 = s->solver == TY_KSOLVE_CG32_REFINE;
  TY_CU(KD_CALL(h, kdif_residual, m, k, dt, q));
  TY_CU(KD_CALL(h, kdif_assemble, m, k, dt, f32 ? 1 : 0, q));
  double* P = k.pinned;
  const int check = 10;  // iterations between host reads of the residual norm
  if (!f32) {
    // fused single-reduction CG; the mixed form runs on the FP32 conductances until the
    // residual is below kSwitch, then restarts on the FP64 conductances from the FP64
    // system's residual
    constexpr double kSwitch = 1e-6;
    bool a32 = s->solver == TY_KSOLVE_CG_MIXED && s->tol < kSwitch;
    TY_CU(KD_CALL(h, kdif_ell_build, m, k, dt, q));
    TY_CU(KD_CALL(h, kdif_fcg_a, m, k, 1, q));
    TY_CU(KD_CALL(h, kdif_fcg_b, m, k, 1, a32 ? 1 : 0, q));
    if (int rc = fetch(h, 3, 1)) return rc;
    const double b2 = P[3];
    double rel = 0.0;
    int it = 0;
    if (b2 > 0.0) {
      rel = 1.0;
      while (it < s->max_it) {
        TY_CU(KD_CALL(h, kdif_fcg_a, m, k, 0, q));
        TY_CU(KD_CALL(h, kdif_fcg_b, m, k, 0, a32 ? 1 : 0, q));
        ++it;
        if (it % check == 0 || it == s->max_it) {
          if (int rc = fetch(h, 11, 1)) return rc;
          rel = std::sqrt(P[11] / b2);
          if (a32 && rel < kSwitch) {  // restart on the FP64 matrix from the true residual
            TY_CU(KD_CALL(h, kdif_fcg_replace, m, k, q));
            TY_CU(KD_CALL(h, kdif_fcg_a, m, k, 2, q));
            TY_CU(KD_CALL(h, kdif_fcg_b, m, k, 1, 0, q));
            a32 = false;
            st->refinements = 1;
            continue;
          }
          if (!a32 && rel < s->tol) break;
        }
      }
    }
    st->iterations = it;
    st->rel_res = rel;
  } else {
    TY_CU(cudaMemsetAsync(k.x, 0, m.nci * sizeof(double), q));
    const double inner = s->inner_tol > 0.0 ? s->inner_tol : 1e-5;
    double b2 = -1.0, rel = 1.0;
    int total = 0, outer = 0;
    for (outer = 0; outer < 100; ++outer) {
      TY_CU(KD_CALL(h, kdif_residual64, m, k, q));   // r = b - S x (FP64), r32 = (float) r
      if (int rc = fetch(h, 5, 1)) return rc;
      if (b2 < 0.0) b2 = P[5];
      rel = b2 > 0.0 ? std::sqrt(P[5] / b2) : 0.0;
      if (rel < s->tol) break;
      TY_CU(KD_CALL(h, kdif_cg_start, m, k, 1, q));
      if (int rc = fetch(h, 3, 1)) return rc;
      const double r2 = P[3];
      int it = 0;
      while (it < s->max_it) {
        TY_CU(KD_CALL(h, kdif_cg_iter, m, k, 1, q));
        ++it;
        if (it % check == 0 || it == s->max_it) {
          if (int rc = fetch(h, 4, 1)) return rc;
          if (!(std::sqrt(P[4] / r2) >= inner)) break;
        }
      }
      total += it;
      TY_CU(KD_CALL(h, kdif_refine, m, k, q));       // x += (double) x32
    }
    st->iterations = total;
    st->refinements = outer;
    st->rel_res = rel;
  }
  TY_CU(KD_CALL(h, kdif_update_T, m, k, q));
  TY_CU(KD_CALL(h, imp_asum, k.x, (size_t)m.nci, k.part, k.scal + 6, q));
  if (int rc = fetch(h, 6, 1)) return rc;
  st->du_l1 = P[6];
  return TY_OK;
}

int ty_kdif_fourier_dt(ty_mesh* h, double fourier, double* dt) {
  if (int rc = kd_ready(h)) return rc;
  if (!dt || !(fourier > 0.0)) return TY_ERR_ARG;
  const int nci = h->m.nci, nfi = h->m.nfi, nf = h->m.nf;
  std::vector<double> s2(nci, 0.0);
  for (int f = 0; f < nfi; ++f) {
    const double a = h->fsurf[f] * h->fsurf[f];
    s2[h->fc1[f]] = s2[h->fc1[f]] + a;
    s2[h->fc2[f]] = s2[h->fc2[f]] + a;
  }
  for (int f = nfi; f < nf; ++f) s2[h->fc1[f]] = s2[h->fc1[f]] + h->fsurf[f] * h->fsurf[f];
  double best = std::numeric_limits<double>::max();
  for (int c = 0; c < nci; ++c) {
    const double v = h->cvol[c];
    double x = 2.0 * fourier * (v * v) / s2[c];
    x = x * h->kd.cp / h->kd_k[c];
    best = std::min(best, x);
  }
  *dt = best;
  return TY_OK;
}

int ty_kdif_get(ty_mesh* h, int32_t which, double* out) {
  if (int rc = kd_ready(h)) return rc;
  if (!out) return TY_ERR_ARG;
  const DevMesh& m = h->m;
  const KdifState& k = h->kd;
  TY_CU(cudaStreamSynchronize(h->stream));
  switch (which) {
    case 0: TY_CU(cudaMemcpy(out, k.T, m.nc * sizeof(double), cudaMemcpyDeviceToHost)); return TY_OK;
    case 1:
      for (int d = 0; d < 3; ++d)
        TY_CU(cudaMemcpy(out + (size_t)d * m.nci, k.grad + (size_t)d * m.ldc, m.nci * sizeof(double),
                         cudaMemcpyDeviceToHost));
      return TY_OK;
    case 2: TY_CU(cudaMemcpy(out, k.flux, m.nf * sizeof(double), cudaMemcpyDeviceToHost)); return TY_OK;
    case 3: TY_CU(cudaMemcpy(out, k.jac, m.nf * sizeof(double), cudaMemcpyDeviceToHost)); return TY_OK;
    case 4: TY_CU(cudaMemcpy(out, k.diag, m.nci * sizeof(double), cudaMemcpyDeviceToHost)); return TY_OK;
    case 5: TY_CU(cudaMemcpy(out, k.bal, m.nci * sizeof(double), cudaMemcpyDeviceToHost)); return TY_OK;
    default: return TY_ERR_ARG;
  }
}

int ty_kdif_matvec(ty_mesh* h, const double* x, double* y) {
  if (int rc = kd_ready(h)) return rc;
  if (!x || !y) return TY_ERR_ARG;
  const size_t n = h->m.nci;
  TY_CU(cudaMemcpyAsync(h->kd.p, x, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  TY_CU(KD_CALL(h, kdif_matvec, h->m, h->kd, h->kd.p, h->kd.q, h->stream));
  TY_CU(cudaMemcpyAsync(y, h->kd.q, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TY_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

}  // extern "C"
