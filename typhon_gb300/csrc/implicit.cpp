// Implicit step of libtyphon_gpu: ty_implicit_step and its debug accessors.
//
// One call is one backward-Euler step of Typhon's implicit method (TIME_PARAM METHOD =
// IMPLICIT), i.e. what calc_rhs.f90:121-138 does with calc_jacobian set, followed by
// update_field.f90:38:
//   1. stability time step per cell (calc_ns_timestep.f90), global minimum unless local;
//   2. residual with flux Jacobians (integration_grid.f90:49-116), BDLU assembly
//      (build_implicit_bdlu.f90:44-83), ghost rows of the right-hand side zeroed
//      (build_implicit.f90:66-74);
//   3. linear solve (implicit_solve.f90:39-86), then U += dU.
// Solvers of step 3:
//   TY_KRYLOV_GMRES   Typhon's bdlu_gmres (SOURCE/MATH/bdlu_gmres.f90:50-217): restarted
//                     GMRES(NKRYLOV), modified Gram-Schmidt, Givens rotations, x0 = b/diag,
//                     its stopping test and restart limit, no preconditioner, FP64.
//   TY_KRYLOV_FGMRES  flexible GMRES(m) with right block-Jacobi preconditioning on the
//                     assembled BDLU matrix (new), its basis orthogonalised through a measured
//                     Gram matrix; FP64, or mixed: FP32 blocks, FP32 mat-vec and preconditioner,
//                     with the basis in FP64 (TY_PREC_MIXED_FP64ORTHO) or in FP32
//                     (TY_PREC_MIXED); residuals, Hessenberg algebra and update in FP64.
//   TY_KRYLOV_JFNK    the same flexible GMRES with Jacobian-free products
//                     J z = z - (R(U + eps z) - R(U)) / eps of the full FP64 residual,
//                     block-Jacobi preconditioned with the assembled diagonal blocks (new;
//                     Typhon's gmres_free.f90 is not called by its drivers).
// The Hessenberg matrix, the Givens rotations and the small triangular solve run on the host
// from the device dot products (one device-to-host copy of a column per Krylov vector).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>

#include "handle.hpp"

using namespace tyk;
using namespace tyi;

#define IMP_CALL(h, fn, ...) \
  ((h)->o.mode == TY_MODE_FAST ? tyk::kfast::fn(__VA_ARGS__) : tyk::kexact::fn(__VA_ARGS__))
#define IMP_CU(expr)                                         \
  do {                                                       \
    cudaError_t e_ = (expr);                                 \
    if (e_ != cudaSuccess) return cuda_fail(e_, #expr);      \
  } while (0)

namespace {

constexpr int kScalGram = 0;                  // scal offsets of the flexible GMRES: V^T v_j, v_j . v_j
constexpr int kScalProj = kMaxCgs + 1;        // V^T w, w . w (both fetched in one copy)
constexpr int kScalCoef = 2 * kMaxCgs + 4;    // c of the next basis vector v_j, then 1 / nu at + j (one copy)
constexpr int kScalY = 2 * kMaxKrylov + 4;    // solution coefficients (kMaxKrylov)
constexpr int kScalMisc = 3 * kMaxKrylov + 4; // reductions of the step (16)
constexpr int kScalCount = 3 * kMaxKrylov + 20;

template <class T>
int grow(ty_mesh* h, T*& p, size_t n) {
  if (p) {
    auto it = std::find(h->allocs.begin(), h->allocs.end(), (void*)p);
    if (it != h->allocs.end()) h->allocs.erase(it);
    cudaFree(p);
    p = nullptr;
  }
  return h->alloc(p, n);
}

// face lists of each interior cell in ascending face order (the order of Typhon's face loops)
int build_lists(ty_mesh* h) {
  ImpState& im = h->imp;
  const DevMesh& m = h->m;
  const int nci = m.nci, ns = m.nslot;
  std::vector<std::vector<int>> l(nci);
  for (int f = 0; f < m.nf; ++f) {
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
  int rc;
  if ((rc = h->alloc(im.cfo, cfo.size())) || (rc = h->alloc(im.cfon, cfon.size())) ||
      (rc = h->alloc(im.dtloc, (size_t)nci)) || (rc = h->alloc(im.jacL, (size_t)m.nf * kBlk)) ||
      (rc = h->alloc(im.jacR, (size_t)m.nf * kBlk)) || (rc = h->alloc(im.b, 5 * (size_t)nci)) ||
      (rc = h->alloc(im.x, 5 * (size_t)nci)) || (rc = h->alloc(im.r, 5 * (size_t)nci)) ||
      (rc = h->alloc(im.w, 5 * (size_t)nci)) || (rc = h->alloc(im.part, (size_t)(kMaxKrylov + 1) * kRedBlocks)) ||
      (rc = h->alloc(im.scal, (size_t)kScalCount)) || (rc = h->alloc(im.done, 1)))
    return rc;
  IMP_CU(cudaMemset(im.done, 0, sizeof(unsigned)));
  IMP_CU(cudaMemcpy(im.cfo, cfo.data(), cfo.size() * sizeof(int), cudaMemcpyHostToDevice));
  IMP_CU(cudaMemcpy(im.cfon, cfon.data(), cfon.size() * sizeof(int), cudaMemcpyHostToDevice));
  if (!im.pinned && cudaMallocHost((void**)&im.pinned, kScalCount * sizeof(double)) != cudaSuccess)
    return TY_ERR_NOMEM;
  im.lists = true;
  return TY_OK;
}

int ensure_buffers(ty_mesh* h, const ty_imp_params* p) {
  ImpState& im = h->imp;
  const DevMesh& m = h->m;
  int rc;
  if (!im.lists && (rc = build_lists(h))) return rc;
  const bool need32 = p->krylov == TY_KRYLOV_FGMRES && p->precision != TY_PREC_FP64;  // FP32 blocks
  const bool need64 = !need32;
  const bool basis32 = p->krylov == TY_KRYLOV_FGMRES && p->precision == TY_PREC_MIXED;  // FP32 basis
  if (need64 && !im.fp64_blocks) {
    if ((rc = h->alloc(im.upper, (size_t)std::max(m.nfi, 1) * kBlk)) ||
        (rc = h->alloc(im.lower, (size_t)std::max(m.nfi, 1) * kBlk)) ||
        (rc = h->alloc(im.diag, (size_t)m.nci * kBlk)) || (rc = h->alloc(im.dinv, (size_t)m.nci * kBlk)))
      return rc;
    im.fp64_blocks = true;
  }
  if (need32 && !im.fp32_blocks) {
    if ((rc = h->alloc(im.upper32, (size_t)std::max(m.nfi, 1) * kBlk32)) ||
        (rc = h->alloc(im.lower32, (size_t)std::max(m.nfi, 1) * kBlk32)) ||
        (rc = h->alloc(im.diag32, (size_t)m.nci * kBlk32)) || (rc = h->alloc(im.dinv32, (size_t)m.nci * kBlk32)))
      return rc;
    im.fp32_blocks = true;
  }
  const size_t n = 5 * (size_t)m.nci;
  const int nk = p->krylov == TY_KRYLOV_BICGSTAB ? std::max(p->nkrylov, 5) : p->nkrylov;
  const bool gm = p->krylov == TY_KRYLOV_GMRES || p->krylov == TY_KRYLOV_BICGSTAB;  // no preconditioned basis
  // Krylov storage: V (FP64 basis, always), V32 (FP32 basis), Z / Z32 (preconditioned vectors
  // of the flexible GMRES in FP64 / FP32); buffers that exist are regrown with the capacity
  if (im.nk < nk || (need32 && !im.Z32) || (basis32 && !im.V32) || (!need32 && !gm && !im.Z)) {
    const int cap = std::max(nk, im.nk);
    if ((rc = grow(h, im.V, (size_t)(cap + 1) * n))) return rc;
    if ((need32 || im.Z32) && (rc = grow(h, im.Z32, (size_t)cap * n))) return rc;
    if ((basis32 || im.V32) && (rc = grow(h, im.V32, (size_t)(cap + 1) * n))) return rc;
    if (((!need32 && !gm) || im.Z) && (rc = grow(h, im.Z, (size_t)cap * n))) return rc;
    im.nk = cap;
  }
  if ((p->krylov == TY_KRYLOV_FGMRES || p->krylov == TY_KRYLOV_JFNK) && !im.bs && (rc = h->alloc(im.bs, n)))
    return rc;
  if (p->krylov == TY_KRYLOV_JFNK && !im.jfnk) {
    if ((rc = h->alloc(im.upert, 5 * (size_t)m.ldc)) || (rc = h->alloc(im.r0, n))) return rc;
    IMP_CU(cudaMemset(im.upert, 0, 5 * (size_t)m.ldc * sizeof(double)));
    im.jfnk = true;
  }
  return TY_OK;
}

constexpr Row5 kOnes{{1.0, 1.0, 1.0, 1.0, 1.0}};
Row5 row_scale(const ImpState& im) {
  Row5 r;
  for (int v = 0; v < 5; ++v) r.v[v] = im.rs[v];
  return r;
}

// copy k device scalars from scal[off..] to the pinned buffer and wait
int fetch(ty_mesh* h, int off, int k) {
  IMP_CU(cudaMemcpyAsync(h->imp.pinned + off, h->imp.scal + off, k * sizeof(double), cudaMemcpyDeviceToHost,
                         h->stream));
  IMP_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}
int put(ty_mesh* h, int off, const double* v, int k) {
  std::memcpy(h->imp.pinned + off, v, k * sizeof(double));
  IMP_CU(cudaMemcpyAsync(h->imp.scal + off, h->imp.pinned + off, k * sizeof(double), cudaMemcpyHostToDevice,
                         h->stream));
  return TY_OK;
}

// ---- Typhon's bdlu_bicgstab on the device (bdlu_bicgstab.f90:40-80) ----
// r1 = im.r, and r2, p, v, s, t in the first five Krylov vectors
int bicgstab_typhon(ty_mesh* h, const ty_imp_params* p, ty_imp_stats* st) {
  ImpState& im = h->imp;
  const DevMesh& m = h->m;
  const size_t n = 5 * (size_t)m.nci;
  cudaStream_t s = h->stream;
  double* P = im.pinned;
  auto V = [&](int i) { return im.V + (size_t)i * n; };
  double* sc = im.scal + kScalMisc + 4;  // 8 device scalars
  IMP_CU(IMP_CALL(h, imp_x0_diag, m, im, im.b, im.x, s));
  IMP_CU(IMP_CALL(h, imp_asum, im.x, n, im.part, im.scal + kScalMisc, s));
  if (int rc = fetch(h, kScalMisc, 1)) return rc;
  const double ref = P[kScalMisc];
  IMP_CU(IMP_CALL(h, imp_matvec, m, im, im.x, im.b, im.r, s, &h->prof));  // r1 = b - A x0
  IMP_CU(cudaMemcpyAsync(V(0), im.r, n * sizeof(double), cudaMemcpyDeviceToDevice, s));  // r2 = r1
  double err = DBL_MAX;
  int nit = 0, matvecs = 1;
  while (err >= ref * p->inv_res && nit <= p->max_it) {
    IMP_CU(IMP_CALL(h, imp_bicgstab_iter, m, im, im.x, im.r, V(0), V(1), V(2), V(3), V(4), nit == 0 ? 1 : 0,
                    im.part, sc, s, &h->prof));
    matvecs += 2;
    if (int rc = fetch(h, kScalMisc + 4 + 7, 1)) return rc;
    err = P[kScalMisc + 4 + 7];
    ++nit;
    if (!(err == err)) break;  // a breakdown (zero r2.v or t.t): stop with the iterate reached
  }
  st->info = nit <= p->max_it ? nit - 1 : -1;
  st->restarts = nit;
  st->matvecs = matvecs;
  IMP_CU(IMP_CALL(h, imp_matvec, m, im, im.x, im.b, im.r, s, &h->prof));
  IMP_CU(IMP_CALL(h, imp_dot, im.r, im.r, n, im.part, im.scal + kScalMisc, s));
  IMP_CU(IMP_CALL(h, imp_dot, im.b, im.b, n, im.part, im.scal + kScalMisc + 1, s));
  if (int rc = fetch(h, kScalMisc, 2)) return rc;
  st->lin_res = P[kScalMisc + 1] > 0.0 ? std::sqrt(P[kScalMisc] / P[kScalMisc + 1]) : 0.0;
  return TY_OK;
}

// ---- Typhon's bdlu_gmres on the device (bdlu_gmres.f90:50-217) ----
int gmres_typhon(ty_mesh* h, const ty_imp_params* p, ty_imp_stats* st) {
  ImpState& im = h->imp;
  const DevMesh& m = h->m;
  const size_t n = 5 * (size_t)m.nci;
  const int nk = p->nkrylov;
  cudaStream_t s = h->stream;
  double* P = im.pinned;
  auto V = [&](int i) { return im.V + (size_t)i * n; };
  std::vector<double> qc(nk + 1), qs(nk + 1), ss(nk + 2), yy(nk + 1), hh((size_t)(nk + 2) * (nk + 1));
  auto H = [&](int i, int j) -> double& { return hh[(size_t)i * (nk + 1) + j]; };  // 1-based
  IMP_CU(IMP_CALL(h, imp_x0_diag, m, im, im.b, im.x, s));
  IMP_CU(IMP_CALL(h, imp_asum, im.x, n, im.part, im.scal + kScalMisc, s));
  IMP_CU(IMP_CALL(h, imp_dot, im.b, im.b, n, im.part, im.scal + kScalMisc + 1, s));
  if (int rc = fetch(h, kScalMisc, 2)) return rc;
  const double ref = P[kScalMisc], normp1 = std::sqrt(P[kScalMisc + 1]);
  const double eps = std::numeric_limits<double>::epsilon();
  double errgmres = DBL_MAX;
  int nit = 0, matvecs = 0;
  while (errgmres >= ref * p->inv_res && nit <= p->max_it * 2) {
    IMP_CU(IMP_CALL(h, imp_matvec, m, im, im.x, im.b, im.r, s, &h->prof));
    ++matvecs;
    IMP_CU(IMP_CALL(h, imp_dot, im.r, im.r, n, im.part, im.scal + kScalMisc, s));
    if (int rc = fetch(h, kScalMisc, 1)) return rc;
    const double beta = std::sqrt(P[kScalMisc]);
    double fact = 1.0 / beta;
    IMP_CU(IMP_CALL(h, imp_scale, im.r, fact, V(0), n, s));
    std::fill(ss.begin(), ss.end(), 0.0);
    ss[1] = beta;
    std::fill(hh.begin(), hh.end(), 0.0);
    int jk;
    for (jk = 1; jk <= nk; ++jk) {
      IMP_CU(IMP_CALL(h, imp_matvec, m, im, V(jk - 1), nullptr, im.w, s, &h->prof));
      ++matvecs;
      for (int ik = 1; ik <= jk; ++ik)  // h(ik,jk) = (w, v_ik) after w -= h(ik-1,jk) v_(ik-1)
        IMP_CU(IMP_CALL(h, imp_mgs_pass, ik > 1 ? V(ik - 2) : nullptr, im.scal + std::max(ik - 2, 0), im.w, V(ik - 1), n,
                        im.part, im.scal + ik - 1, s));
      IMP_CU(IMP_CALL(h, imp_mgs_pass, V(jk - 1), im.scal + jk - 1, im.w, nullptr, n, im.part, im.scal + jk, s));
      if (int rc = fetch(h, 0, jk + 1)) return rc;
      for (int ik = 1; ik <= jk; ++ik) H(ik, jk) = P[ik - 1];
      H(jk + 1, jk) = std::sqrt(P[jk]);
      for (int ik = 1; ik <= jk - 1; ++ik) {
        double tmp = H(ik, jk);
        H(ik, jk) = qc[ik] * tmp + qs[ik] * H(ik + 1, jk);
        H(ik + 1, jk) = -qs[ik] * tmp + qc[ik] * H(ik + 1, jk);
      }
      if (H(jk + 1, jk) > eps * 10 * normp1) {
        if (jk < nk) {
          fact = 1.0 / H(jk + 1, jk);
          IMP_CU(IMP_CALL(h, imp_scale, im.w, fact, V(jk), n, s));
        }
        if (H(jk, jk) == 0) break;
        double tmp = std::sqrt(H(jk, jk) * H(jk, jk) + H(jk + 1, jk) * H(jk + 1, jk));
        qc[jk] = H(jk, jk) / tmp;
        qs[jk] = H(jk + 1, jk) / tmp;
        H(jk, jk) = tmp;
        H(jk + 1, jk) = 0.0;
        ss[jk + 1] = -qs[jk] * ss[jk];
        ss[jk] = qc[jk] * ss[jk];
        if (std::fabs(ss[jk + 1]) < p->inv_res * std::fabs(ss[1])) break;
      } else {
        break;
      }
    }
    const int nkk = std::min(jk, nk);
    for (int j = nkk; j >= 1; --j) {
      double tmp = ss[j];
      for (int ik = j + 1; ik <= nkk; ++ik) tmp = tmp - H(j, ik) * yy[ik];
      yy[j] = tmp / H(j, j);
    }
    if (int rc = put(h, kScalY, &yy[1], nkk)) return rc;
    IMP_CU(IMP_CALL(h, imp_axpy_multi, im.x, im.V, nullptr, n, nkk, im.scal + kScalY, 1, n, s));
    IMP_CU(IMP_CALL(h, imp_matvec, m, im, im.x, im.b, im.r, s, &h->prof));
    ++matvecs;
    IMP_CU(IMP_CALL(h, imp_dot, im.r, im.r, n, im.part, im.scal + kScalMisc, s));
    if (int rc = fetch(h, kScalMisc, 1)) return rc;
    ss[nkk + 1] = std::sqrt(P[kScalMisc]);
    errgmres = ss[nkk + 1] / normp1;
    nit = nit + 1;
  }
  st->restarts = nit;
  st->matvecs = matvecs;
  st->lin_res = errgmres;
  st->info = nit <= p->max_it ? nit - 1 : -1;
  return TY_OK;
}

// ---- flexible GMRES(m), CGS2, right block-Jacobi preconditioning ----
struct Operator {
  ty_mesh* h;
  int kind;  // 0 assembled FP64, 1 assembled FP32 (FP32 basis), 2 Jacobian-free, 3 assembled FP32 (FP64 basis)
  double unorm = 0.0;
  ImpArgs a{};
  int apply(const double* z, const float* z32, double* w, int* matvecs);
};

int Operator::apply(const double* z, const float* z32, double* w, int* matvecs) {
  ImpState& im = h->imp;
  const DevMesh& m = h->m;
  const size_t n = 5 * (size_t)m.nci;
  cudaStream_t s = h->stream;
  ++*matvecs;
  if (kind == 0) {
    IMP_CU(IMP_CALL(h, imp_matvec, m, im, z, nullptr, w, s, &h->prof));
    return TY_OK;
  }
  if (kind == 1 || kind == 3) {
    IMP_CU(IMP_CALL(h, imp_matvec32, m, im, z32, w, s, &h->prof));
    return TY_OK;
  }
  // J z = z - (R(U + eps z) - R(U)) / eps, eps = sqrt(machine eps) (1 + |U|) / |z|
  IMP_CU(IMP_CALL(h, imp_dot, z, z, n, im.part, im.scal + kScalMisc + 8, s));
  if (int rc = fetch(h, kScalMisc + 8, 1)) return rc;
  const double zn = std::sqrt(h->imp.pinned[kScalMisc + 8]);
  if (!(zn > 0.0)) {
    IMP_CU(cudaMemsetAsync(w, 0, n * sizeof(double), s));
    return TY_OK;
  }
  const double eps = std::sqrt(std::numeric_limits<double>::epsilon()) * (1.0 + unorm) / zn;
  IMP_CU(IMP_CALL(h, imp_perturb, m, h->s.u0, z, eps, im.upert, s));
  IMP_CU(MODE_CALL(h, prim_from, h->m, h->s, h->o, im.upert, s, &h->prof));
  if (int rc = stage_faces(h)) return rc;
  IMP_CU(IMP_CALL(h, imp_rhs, m, h->s, im, a, im.r, s));
  IMP_CU(IMP_CALL(h, imp_fd_combine, z, nullptr, im.r, im.r0, 1.0 / eps, row_scale(im), w, n, s));
  return TY_OK;
}

// Restarted flexible GMRES with a block-Jacobi preconditioner and one host synchronisation per
// Krylov vector.  The basis V is not forced to be orthonormal; its Gram matrix G = R^T R is
// measured instead.  Iteration j:
//   1. v_j = (w_{j-1} - V c) / nu (v_0 = r / beta), stored, with its Gram column V^T v_j,
//      v_j . v_j, in one sweep over the basis;
//   2. z_j = M^-1 v_j, w_j = A z_j;
//   3. V^T w_j and w_j . w_j in a second sweep, then on the host c = G^-1 V^T w_j, so that
//      w_j - V c is orthogonal to the basis in exact arithmetic whatever V's rounding, and
//      nu^2 = |w_j|^2 - |R^-T V^T w_j|^2.
// A z_j = V c + nu v_{j+1} holds for the stored vectors, and |V (beta e1 - H y)| =
// |R (beta e1 - H y)|: Givens rotations of R H minimise the true residual norm.  The Gram
// column of v_{j+1} is only measured in the next iteration, so column j of R H is first
// rotated with v_{j+1} taken as orthonormal and rotated again one iteration later.  A
// cancellation of nu^2 below 1e-12 |w_j|^2 means the Krylov space is invariant to working
// precision (breakdown; 1e-10 for the FP32 basis of the mixed solve, whose sweeps run in FP32
// arithmetic): the cycle ends there.
int fgmres(ty_mesh* h, Operator& op, const ty_imp_params* p, ty_imp_stats* st) {
  ImpState& im = h->imp;
  const DevMesh& m = h->m;
  const size_t n = 5 * (size_t)m.nci;
  const int mk = p->nkrylov;
  const bool f32 = op.kind == 1;                    // FP32 basis, swept in FP32 arithmetic
  const bool z32 = op.kind == 1 || op.kind == 3;    // FP32 preconditioned vectors and mat-vec
  cudaStream_t s = h->stream;
  double* P = im.pinned;
  double* V64 = f32 ? nullptr : im.V;
  float* V32 = f32 ? im.V32 : nullptr;
  auto Vd = [&](int i) { return V64 ? V64 + (size_t)i * n : nullptr; };
  auto Vf = [&](int i) { return V32 ? V32 + (size_t)i * n : nullptr; };
  auto Z = [&](int i) { return z32 ? nullptr : im.Z + (size_t)i * n; };
  auto Z32 = [&](int i) { return z32 ? im.Z32 + (size_t)i * n : nullptr; };
  const int ld = mk + 1;
  std::vector<double> R((size_t)ld * ld, 0.0), Hc((size_t)ld * mk, 0.0), T((size_t)ld * mk, 0.0);
  std::vector<double> cs(mk), sn(mk), a(mk + 1), gr(mk), y(mk), u(mk + 1), c(mk + 1), t(mk + 2);
  auto Rm = [&](int i, int j) -> double& { return R[(size_t)i * ld + j]; };
  auto Hm = [&](int i, int j) -> double& { return Hc[(size_t)i * mk + j]; };
  auto Tm = [&](int i, int j) -> double& { return T[(size_t)i * mk + j]; };
  // column jc of R H (R's column jc + 1 measured, or taken as e_{jc+1}), rotated by the
  // earlier rotations; then its own rotation and the rotated right-hand side
  auto rotate_column = [&](int jc, bool measured) {
    for (int i = 0; i <= jc + 1; ++i) {
      double v = 0.0;
      for (int l = i; l <= jc; ++l) v += Rm(i, l) * Hm(l, jc);
      v += (measured ? Rm(i, jc + 1) : (i == jc + 1 ? 1.0 : 0.0)) * Hm(jc + 1, jc);
      t[i] = v;
    }
    for (int i = 0; i < jc; ++i) {
      const double q = cs[i] * t[i] + sn[i] * t[i + 1];
      t[i + 1] = -sn[i] * t[i] + cs[i] * t[i + 1];
      t[i] = q;
    }
    const double den = std::hypot(t[jc], t[jc + 1]);
    cs[jc] = den > 0.0 ? t[jc] / den : 1.0;
    sn[jc] = den > 0.0 ? t[jc + 1] / den : 0.0;
    t[jc] = den;
    for (int i = 0; i <= jc; ++i) Tm(i, jc) = t[i];
    gr[jc] = cs[jc] * a[jc];
    a[jc + 1] = -sn[jc] * a[jc];
  };
  IMP_CU(cudaMemsetAsync(im.x, 0, n * sizeof(double), s));
  IMP_CU(IMP_CALL(h, imp_fd_combine, im.b, nullptr, nullptr, nullptr, 0.0, row_scale(im), im.bs, n, s));
  IMP_CU(IMP_CALL(h, imp_dot, im.bs, im.bs, n, im.part, im.scal + kScalMisc, s));
  if (int rc = fetch(h, kScalMisc, 1)) return rc;
  const double beta0 = std::sqrt(P[kScalMisc]);
  const char* tv = std::getenv("TY_IMPLICIT_TRACE");  // Arnoldi history on stderr when set to 1
  const bool trace = tv && tv[0] == '1';
  int matvecs = 0, cycles = 0;
  double rel = beta0 > 0.0 ? 1.0 : 0.0;
  if (beta0 > 0.0) {
    const double tol = p->inv_res * beta0;
    for (cycles = 0; cycles < std::max(p->max_it, 1); ++cycles) {
      double beta;
      const double* src = im.bs;
      if (cycles == 0) {
        beta = beta0;
      } else {  // r = b - A x
        if (z32) IMP_CU(IMP_CALL(h, imp_to_f32, im.x, Z32(0), n, s));
        if (int rc = op.apply(im.x, Z32(0), im.w, &matvecs)) return rc;
        IMP_CU(IMP_CALL(h, imp_fd_combine, im.bs, nullptr, im.w, nullptr, 1.0, kOnes, im.r, n, s));
        IMP_CU(IMP_CALL(h, imp_dot, im.r, im.r, n, im.part, im.scal + kScalMisc, s));
        if (int rc = fetch(h, kScalMisc, 1)) return rc;
        beta = std::sqrt(P[kScalMisc]);
        rel = beta / beta0;
        if (beta <= tol) break;
        src = im.r;
      }
      const double binv = 1.0 / beta;
      if (int rc = put(h, kScalCoef, &binv, 1)) return rc;
      a[0] = beta;
      int j, nused = 0;
      for (j = 0; j < mk; ++j) {
        IMP_CU(IMP_CALL(h, imp_basis_pass, V64, V32, n, j, im.scal + kScalCoef, j == 0 ? src : im.w,
                        im.scal + kScalCoef + j, 1, n, im.part, im.done, im.scal + kScalGram, s, &h->prof));
        IMP_CU(IMP_CALL(h, imp_precond, m, im, Vd(j), Vf(j), Z(j), Z32(j), s, &h->prof));
        if (int rc = op.apply(Z(j), Z32(j), im.w, &matvecs)) return rc;
        IMP_CU(IMP_CALL(h, imp_basis_pass, V64, V32, n, j + 1, nullptr, im.w, nullptr, 0, n, im.part, im.done,
                        im.scal + kScalProj, s, &h->prof));
        if (int rc = fetch(h, 0, kScalProj + j + 2)) return rc;
        // column j of the Cholesky factor of G
        double d = P[kScalGram + j];
        for (int i = 0; i < j; ++i) {
          double v = P[kScalGram + i];
          for (int l = 0; l < i; ++l) v -= Rm(l, i) * Rm(l, j);
          Rm(i, j) = v / Rm(i, i);
          d -= Rm(i, j) * Rm(i, j);
        }
        if (!(d > 1e-10 * P[kScalGram + j])) break;  // v_j no longer independent of the basis
        Rm(j, j) = std::sqrt(d);
        if (j == 0) a[0] = beta * Rm(0, 0);
        else rotate_column(j - 1, true);
        // c = G^-1 V^T w: R^T u = V^T w, R c = u
        const double ww = P[kScalProj + j + 1];
        double uu = 0.0;
        for (int i = 0; i <= j; ++i) {
          double v = P[kScalProj + i];
          for (int l = 0; l < i; ++l) v -= Rm(l, i) * u[l];
          u[i] = v / Rm(i, i);
          uu += u[i] * u[i];
        }
        for (int i = j; i >= 0; --i) {
          double v = u[i];
          for (int l = i + 1; l <= j; ++l) v -= Rm(i, l) * c[l];
          c[i] = v / Rm(i, i);
        }
        const double nu2 = ww - uu;
        const bool invariant = !(nu2 > (f32 ? 1e-10 : 1e-12) * ww);
        const double nu = invariant ? 0.0 : std::sqrt(nu2);
        for (int i = 0; i <= j; ++i) Hm(i, j) = c[i];
        Hm(j + 1, j) = nu;
        rotate_column(j, false);
        nused = j + 1;
        if (trace)
          std::fprintf(stderr, "ty_implicit fgmres cycle %d j %d r_jj %.6e nu %.6e |g|/|b| %.6e\n", cycles, j,
                       Rm(j, j), nu, std::fabs(a[j + 1]) / beta0);
        if (std::fabs(a[j + 1]) <= tol || invariant) break;
        c[j + 1] = 1.0 / nu;  // c of v_{j+1}, then its scale, in one copy
        if (int rc = put(h, kScalCoef, c.data(), j + 2)) return rc;
      }
      for (int i = nused - 1; i >= 0; --i) {
        double v = gr[i];
        for (int k = i + 1; k < nused; ++k) v -= Tm(i, k) * y[k];
        y[i] = v / Tm(i, i);
      }
      if (nused > 0) {
        if (int rc = put(h, kScalY, y.data(), nused)) return rc;
        IMP_CU(IMP_CALL(h, imp_axpy_multi, im.x, z32 ? nullptr : im.Z, z32 ? im.Z32 : nullptr, n, nused,
                        im.scal + kScalY, 0, n, s));
      }
      rel = std::fabs(a[nused]) / beta0;
      if (std::fabs(a[nused]) <= tol) { ++cycles; break; }
    }
  }
  st->restarts = cycles;
  st->matvecs = matvecs;
  st->lin_res = rel;
  st->info = rel <= p->inv_res ? cycles - 1 : -1;
  return TY_OK;
}

}  // namespace

extern "C" {

int ty_implicit_step(ty_mesh* h, const ty_imp_params* p, ty_imp_stats* st) {
  if (!p || !st) return TY_ERR_ARG;
  if (int rc = ready(h)) return rc;
  if (p->krylov < TY_KRYLOV_GMRES || p->krylov > TY_KRYLOV_BICGSTAB || p->precision < TY_PREC_FP64 ||
      p->precision > TY_PREC_MIXED_FP64ORTHO || p->nkrylov < 1 || p->max_it < 0 || !(p->inv_res > 0.0) || !(p->cfl > 0.0) ||
      ((p->krylov == TY_KRYLOV_GMRES || p->krylov == TY_KRYLOV_BICGSTAB) && p->nkrylov > kMaxKrylov) ||
      ((p->krylov == TY_KRYLOV_FGMRES || p->krylov == TY_KRYLOV_JFNK) && p->nkrylov > kMaxCgs) ||
      (p->krylov != TY_KRYLOV_FGMRES && p->precision != TY_PREC_FP64) ||
      (p->scaling != TY_IMP_SCALE_STATE && p->scaling != TY_IMP_SCALE_NONE)) {
    tyi::set_error("ty_imp_params: option out of range (GMRES: nkrylov <= 64, FP64; FGMRES/JFNK: nkrylov <= 32)");
    return TY_ERR_ARG;
  }
  if (h->o.scheme == TY_SCH_AUSMM) {  // calc_flux_ausmm.f90:121-137: no AUSM-M Jacobian in Typhon
    tyi::set_error("ty_implicit_step: the AUSM-M flux has no Jacobian");
    return TY_ERR_UNSUPPORTED;
  }
  std::memset(st, 0, sizeof(*st));
  int rc;
  if ((rc = ensure_buffers(h, p))) return rc;
  ImpState& im = h->imp;
  const DevMesh& m = h->m;
  DevState& S = h->s;
  cudaStream_t s = h->stream;
  const size_t n = 5 * (size_t)m.nci;
  // 1. time step
  if ((rc = set_dt_slot(h, 0, DBL_MAX))) return rc;
  IMP_CU(IMP_CALL(h, imp_dtloc, m, S, h->o, im, p->cfl, S.dtbits, s));
  if ((rc = check_err(h))) return rc;
  // 2. residual, Jacobians, assembly
  if ((rc = ensure_prim(h))) return rc;
  if ((rc = stage_faces(h))) return rc;
  ImpArgs a{};
  a.local_dt = p->local_dt ? 1 : 0;
  a.dtg = S.dtbits;
  a.src = (h->o.mode == TY_MODE_FAST && h->o.highres != TY_HRES_NONE) ? 2 : (h->o.postlim != TY_POSTLIM_NONE ? 1 : 0);
  const bool mixed = p->krylov == TY_KRYLOV_FGMRES && p->precision != TY_PREC_FP64;
  a.want64 = mixed ? 0 : 1;
  a.want32 = mixed ? 1 : 0;
  IMP_CU(IMP_CALL(h, imp_assemble, m, S, h->o, im, a, s, &h->prof));
  IMP_CU(IMP_CALL(h, imp_rhs, m, S, im, a, im.b, s));
  if ((rc = check_err(h))) {
    tyi::set_error(std::string("implicit assembly: singular diagonal block (") + tyi::last_error() + ")");
    return rc;
  }
  IMP_CU(IMP_CALL(h, imp_res_norms, m, im, a, im.b, im.part, im.scal + kScalMisc + 2, s));
  IMP_CU(cudaMemcpyAsync(&st->dt_min, S.dtbits, sizeof(double), cudaMemcpyDeviceToHost, s));
  if ((rc = fetch(h, kScalMisc + 2, 5))) return rc;
  im.last_local = a.local_dt;
  im.last_dt = st->dt_min;
  for (int v = 0; v < 5; ++v) st->res_l2[v] = std::sqrt(im.pinned[kScalMisc + 2 + v]);
  // 3. solve.  The flexible GMRES scales equation v of its system by 1 / s_v, s from the
  // state's RMS magnitudes: s_rho, s_rhoE and sqrt(s_rho s_rhoE) for the three momentum
  // components (a momentum density, the same for all three so that the scale is invariant to
  // rotations).  Unscaled, the 2-norm of a low-Mach residual is the energy equation's alone.
  for (int v = 0; v < 5; ++v) im.rs[v] = im.rsi[v] = 1.0;
  if ((p->krylov == TY_KRYLOV_FGMRES || p->krylov == TY_KRYLOV_JFNK) && p->scaling == TY_IMP_SCALE_STATE) {
    IMP_CU(IMP_CALL(h, imp_dot, S.u0, S.u0, (size_t)m.nci, im.part, im.scal + kScalMisc, s));
    IMP_CU(IMP_CALL(h, imp_dot, S.u0 + m.ldc, S.u0 + m.ldc, (size_t)m.nci, im.part, im.scal + kScalMisc + 1, s));
    if ((rc = fetch(h, kScalMisc, 2))) return rc;
    const double sr = std::sqrt(im.pinned[kScalMisc] / m.nci), se = std::sqrt(im.pinned[kScalMisc + 1] / m.nci);
    const double sm = std::sqrt(sr * se);
    if (sr > 0.0 && se > 0.0 && std::isfinite(sr) && std::isfinite(se)) {
      const double sv[5] = {sr, se, sm, sm, sm};
      for (int v = 0; v < 5; ++v) {
        im.rsi[v] = sv[v];
        im.rs[v] = 1.0 / sv[v];
      }
    }
  }
  if (p->krylov == TY_KRYLOV_GMRES) {
    rc = gmres_typhon(h, p, st);
  } else if (p->krylov == TY_KRYLOV_BICGSTAB) {
    rc = bicgstab_typhon(h, p, st);
  } else {
    Operator op{h, mixed ? (p->precision == TY_PREC_MIXED ? 1 : 3) : (p->krylov == TY_KRYLOV_JFNK ? 2 : 0)};
    op.a = a;
    if (op.kind == 2) {
      IMP_CU(cudaMemcpyAsync(im.r0, im.b, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      IMP_CU(IMP_CALL(h, imp_dot, S.u0, S.u0, 5 * (size_t)m.ldc, im.part, im.scal + kScalMisc + 9, s));
      if ((rc = fetch(h, kScalMisc + 9, 1))) return rc;
      op.unorm = std::sqrt(im.pinned[kScalMisc + 9]);
    }
    rc = fgmres(h, op, p, st);
  }
  for (int v = 0; v < 5; ++v) im.rs[v] = im.rsi[v] = 1.0;
  if (rc) return rc;
  // 4. update U += dU
  IMP_CU(IMP_CALL(h, imp_update_state, m, S, im.x, im.part, im.scal + kScalMisc + 10, s));
  if ((rc = fetch(h, kScalMisc + 10, 6))) return rc;
  for (int v = 0; v < 5; ++v) st->du_l1[v] = im.pinned[kScalMisc + 10 + v];
  st->du_mom = im.pinned[kScalMisc + 15];
  h->prim_valid = false;
  return TY_OK;
}

int ty_implicit_get(ty_mesh* h, int32_t which, double* out) {
  if (!h || !out) return TY_ERR_ARG;
  const ImpState& im = h->imp;
  const DevMesh& m = h->m;
  if (!im.lists) { tyi::set_error("no implicit step has run"); return TY_ERR_STATE; }
  IMP_CU(cudaSetDevice(h->device));
  IMP_CU(cudaStreamSynchronize(h->stream));
  auto blocks = [&](const double* src, int nb) -> int {
    if (!src) { tyi::set_error("matrix not assembled in FP64"); return TY_ERR_STATE; }
    std::vector<double> t((size_t)nb * kBlk);
    IMP_CU(cudaMemcpy(t.data(), src, t.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < nb; ++i)
      for (int k = 0; k < 25; ++k) out[25 * (size_t)i + k] = t[(size_t)i * kBlk + k];
    return TY_OK;
  };
  switch (which) {
    case 0: return blocks(im.jacL, m.nf);
    case 1: return blocks(im.jacR, m.nf);
    case 2: return blocks(im.diag, m.nci);
    case 3: return blocks(im.upper, m.nfi);
    case 4: return blocks(im.lower, m.nfi);
    case 5:
      if (im.last_local) IMP_CU(cudaMemcpy(out, im.dtloc, m.nci * sizeof(double), cudaMemcpyDeviceToHost));
      else std::fill(out, out + m.nci, im.last_dt);
      return TY_OK;
    case 6: IMP_CU(cudaMemcpy(out, im.b, 5 * (size_t)m.nci * sizeof(double), cudaMemcpyDeviceToHost)); return TY_OK;
    case 7: IMP_CU(cudaMemcpy(out, im.x, 5 * (size_t)m.nci * sizeof(double), cudaMemcpyDeviceToHost)); return TY_OK;
    default: return TY_ERR_ARG;
  }
}

int ty_implicit_matvec(ty_mesh* h, const double* x, double* y) {
  if (!h || !x || !y) return TY_ERR_ARG;
  ImpState& im = h->imp;
  if (!im.lists || !im.fp64_blocks) { tyi::set_error("no FP64 matrix assembled"); return TY_ERR_STATE; }
  IMP_CU(cudaSetDevice(h->device));
  const size_t n = 5 * (size_t)h->m.nci;
  IMP_CU(cudaMemcpyAsync(im.r, x, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  IMP_CU(IMP_CALL(h, imp_matvec, h->m, im, im.r, nullptr, im.w, h->stream, &h->prof));
  IMP_CU(cudaMemcpyAsync(y, im.w, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  IMP_CU(cudaStreamSynchronize(h->stream));
  return TY_OK;
}

}  // extern "C"
