// Heat-conduction (KDIF) kernels, instantiated once per arithmetic mode after kernels.cuh.
//
// Face flux per unit surface (calc_kdif_flux.f90:106-137, theta = 1) with the face
// conductivity of the two cells, then times S; imposed-flux walls replace it
// (kdif_bocoflux.f90) and have no Jacobian.  The residual gathers the face fluxes in
// colour order (flux_to_res.f90); the diagonal of the symmetrised implicit matrix
// diag(V/dt) A is V/dt - sum_f J_R S over the cell's faces in ascending face order, its
// off-diagonal J_R S, as the oracle assembles them.  Conjugate gradients keep their scalars
// on the device; the host reads the residual norm every few iterations.
#pragma once
#include "implicit.hpp"
#include "kdif.hpp"

namespace tyk {
namespace TY_KNS {

__global__ void __launch_bounds__(kBlock) k_kdif_ghost(DevMesh m, KdifState k) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m.ng) return;
  const int f = m.gface[g];
  k.T[m.nci + g] = k.fkind[f] == TY_KBC_ISOTHERMAL ? k.fval[f] : k.T[m.gsrc[g]];
}

// least-squares gradient of T (the 5-variable k_grad restricted to one scalar)
__global__ void __launch_bounds__(kBlock) k_kdif_grad(DevMesh m, KdifState k) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  double b0 = 0.0, b1 = 0.0, b2 = 0.0;
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = m.cf[sl * (size_t)m.nci + c];
    if (e < 0) break;
    const int f = e >> 1;
    const double dsca = k.T[m.fc2[f]] - k.T[m.fc1[f]];
    if constexpr (kFast) {
      const int side = e & 1;
      b0 = fma(dsca, d3(m.lsqw, m.ldf, f, 3 * side), b0);
      b1 = fma(dsca, d3(m.lsqw, m.ldf, f, 3 * side + 1), b1);
      b2 = fma(dsca, d3(m.lsqw, m.ldf, f, 3 * side + 2), b2);
    } else {
      b0 = b0 + dsca * d3(m.dcg, m.ldf, f, 0);
      b1 = b1 + dsca * d3(m.dcg, m.ldf, f, 1);
      b2 = b2 + dsca * d3(m.dcg, m.ldf, f, 2);
    }
  }
  if constexpr (!kFast) {  // cholesky_solve (MATRIX.f90:79-111)
    const size_t n = m.nci;
    const double L11 = m.lsq[c], L21 = m.lsq[n + c], L31 = m.lsq[2 * n + c];
    const double L22 = m.lsq[3 * n + c], L32 = m.lsq[4 * n + c], L33 = m.lsq[5 * n + c];
    double x1 = b0, x2 = b1, x3 = b2;
    x1 = x1 / L11;
    x2 = x2 - L21 * x1;
    x2 = x2 / L22;
    x3 = x3 - L31 * x1;
    x3 = x3 - L32 * x2;
    x3 = x3 / L33;
    x3 = x3 / L33;
    x2 = x2 - L32 * x3;
    x2 = x2 / L22;
    x1 = x1 - L21 * x2;
    x1 = x1 - L31 * x3;
    x1 = x1 / L11;
    b0 = x1; b1 = x2; b2 = x3;
  }
  const size_t ld = m.ldc;
  k.grad[c] = b0;
  k.grad[ld + c] = b1;
  k.grad[2 * ld + c] = b2;
}

__global__ void __launch_bounds__(kBlock) k_kdif_face(DevMesh m, KdifState k) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const size_t lf = m.ldf, ld = m.ldc;
  const int icl = m.fc1[f], icr = m.fc2[f];
  const double dHL = k.kgeo[f], dHR = k.kgeo[lf + f];
  const double vx = k.kgeo[2 * lf + f], vy = k.kgeo[3 * lf + f], vz = k.kgeo[4 * lf + f];
  const double dn = k.kgeo[5 * lf + f], dl2 = k.kgeo[6 * lf + f];
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  const double kl = k.k[icl], kr = k.k[icr];
  const double kH = kl == kr ? kl : 1.0 / (dHL / kl + dHR / kr);
  const double TL = k.T[icl], TR = k.T[icr];
  double Fl;
  if (k.scheme == TY_KDIF_COMPACT) {
    Fl = -kH * (TR - TL) * dn / dl2;
  } else {
    const double gx = dHL * k.grad[icr] + dHR * k.grad[icl];
    const double gy = dHL * k.grad[ld + icr] + dHR * k.grad[ld + icl];
    const double gz = dHL * k.grad[2 * ld + icr] + dHR * k.grad[2 * ld + icl];
    if (k.scheme == TY_KDIF_CELLAVG) {
      Fl = -kH * (gx * nx + gy * ny + gz * nz);
    } else {
      const double pscal = dn / dl2;
      const double Fcomp = pscal * (TR - TL);
      const double tp = 1.0 * pscal;
      const double wx = nx - tp * vx, wy = ny - tp * vy, wz = nz - tp * vz;
      const double Favg = gx * wx + gy * wy + gz * wz;
      Fl = -kH * (1.0 * Fcomp + Favg);
    }
  }
  double jR = -kH * dn / (k.cp * dl2);
  if (f >= m.nfi && k.fkind[f] == TY_KBC_FLUX) {
    Fl = -k.fval[f];
    jR = 0.0;
  }
  const double S = m.fs[f];
  k.flux[f] = S * Fl;
  k.jac[f] = S * jR;
}

// flux balance sum(+-F S) in colour order; optionally dt/V times it into R
__global__ void __launch_bounds__(kBlock) k_kdif_gather(DevMesh m, KdifState k, double dt, double* __restrict__ R) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  double s = 0.0;
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = m.cf[sl * (size_t)m.nci + c];
    if (e < 0) break;
    const double F = k.flux[e >> 1];
    s = (e & 1) ? s + F : s - F;
  }
  k.bal[c] = s;
  if (R) R[c] = dt / m.cvol[c] * s;
}

__global__ void __launch_bounds__(kBlock) k_kdif_diag(DevMesh m, KdifState k, double dt, int want32) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  double d = m.cvol[c] / dt;
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = k.cfo[sl * (size_t)m.nci + c];
    if (e < 0) break;
    d = d - k.jac[e >> 1];
  }
  k.diag[c] = d;
  if (want32) k.diag32[c] = (float)d;
}

__global__ void k_kdif_jac32(KdifState k, int nf) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) k.jac32[f] = (float)k.jac[f];
}

// y = S x: diagonal, then the cell's interior faces in ascending order; optional partial x.y
template <class V>
__global__ void __launch_bounds__(kRedThreads) k_kdif_mv(DevMesh m, KdifState k, const V* __restrict__ x,
                                                          V* __restrict__ y, const V* __restrict__ dg,
                                                          const V* __restrict__ off, double* __restrict__ part) {
  double acc = 0.0;
  for (int c = blockIdx.x * kRedThreads + threadIdx.x; c < m.nci; c += gridDim.x * kRedThreads) {
    V s = dg[c] * x[c];
    for (int sl = 0; sl < m.nslot; ++sl) {
      const int e = k.cfo[sl * (size_t)m.nci + c];
      if (e < 0) break;
      const int f = e >> 1;
      if (f >= m.nfi) break;
      s = s + off[f] * x[k.cfon[sl * (size_t)m.nci + c]];
    }
    y[c] = s;
    acc += (double)x[c] * (double)s;
  }
  if (part) {
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
  }
}

// CG start: x = 0, z = r / diag, p = z; partial r.z and r.r
template <class V>
__global__ void __launch_bounds__(kRedThreads) k_kdif_cg0(int n, V* x, const V* r, V* z, V* p, const V* dg,
                                                           double* part) {
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * kRedThreads + threadIdx.x; i < n; i += gridDim.x * kRedThreads) {
    const V zi = r[i] / dg[i];
    x[i] = V(0);
    z[i] = zi;
    p[i] = zi;
    rz += (double)r[i] * (double)zi;
    rr += (double)r[i] * (double)r[i];
  }
  rz = block_sum(rz);
  if (threadIdx.x == 0) part[blockIdx.x] = rz;
  rr = block_sum(rr);
  if (threadIdx.x == 0) part[kRedBlocks + blockIdx.x] = rr;
}

// x += alpha p, r -= alpha q, z = r / diag; partial r.z and r.r (alpha = scal[0] / scal[1])
template <class V>
__global__ void __launch_bounds__(kRedThreads) k_kdif_cg1(int n, V* x, V* r, V* z, const V* p, const V* q,
                                                           const V* dg, const double* scal, double* part) {
  const double alpha = scal[0] / scal[1];
  double rz = 0.0, rr = 0.0;
  for (int i = blockIdx.x * kRedThreads + threadIdx.x; i < n; i += gridDim.x * kRedThreads) {
    x[i] = x[i] + V(alpha) * p[i];
    const V ri = r[i] - V(alpha) * q[i];
    r[i] = ri;
    const V zi = ri / dg[i];
    z[i] = zi;
    rz += (double)ri * (double)zi;
    rr += (double)ri * (double)ri;
  }
  rz = block_sum(rz);
  if (threadIdx.x == 0) part[blockIdx.x] = rz;
  rr = block_sum(rr);
  if (threadIdx.x == 0) part[kRedBlocks + blockIdx.x] = rr;
}

// p = z + beta p, beta = scal[2] / scal[0]; then scal[0] = scal[2]
template <class V>
__global__ void k_kdif_cg2(int n, const V* z, V* p, const double* scal) {
  const double beta = scal[2] / scal[0];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = z[i] + V(beta) * p[i];
}

// scalar finals: mode 0 start (scal[0] = rz, scal[3] = scal[4] = rr), mode 1 p.q (scal[1]),
// mode 2 update (scal[2] = rz', scal[4] = rr), mode 3 (after cg2) scal[0] = scal[2]
__global__ void __launch_bounds__(kRedThreads) k_kdif_final(const double* part, int nb, int mode, double* scal) {
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nb; i += kRedThreads) {
    a += part[i];
    if (mode != 1) b += part[kRedBlocks + i];
  }
  a = block_sum(a);
  b = block_sum(b);
  if (threadIdx.x == 0) {
    if (mode == 0) { scal[0] = a; scal[3] = b; scal[4] = b; }
    else if (mode == 1) scal[1] = a;
    else { scal[2] = a; scal[4] = b; }
  }
}
__global__ void k_kdif_shift(double* scal) { scal[0] = scal[2]; }

// r = bal - S x (FP64), r32 = r (the refinement residual)
__global__ void __launch_bounds__(kRedThreads) k_kdif_res64(DevMesh m, KdifState k, double* part) {
  double rr = 0.0;
  for (int c = blockIdx.x * kRedThreads + threadIdx.x; c < m.nci; c += gridDim.x * kRedThreads) {
    double s = k.diag[c] * k.x[c];
    for (int sl = 0; sl < m.nslot; ++sl) {
      const int e = k.cfo[sl * (size_t)m.nci + c];
      if (e < 0) break;
      const int f = e >> 1;
      if (f >= m.nfi) break;
      s = s + k.jac[f] * k.x[k.cfon[sl * (size_t)m.nci + c]];
    }
    const double r = k.bal[c] - s;
    k.r[c] = r;
    k.r32[c] = (float)r;
    rr += r * r;
  }
  rr = block_sum(rr);
  if (threadIdx.x == 0) part[blockIdx.x] = rr;
}
__global__ void __launch_bounds__(kRedThreads) k_kdif_final1(const double* part, int nb, double* out) {
  double a = 0.0;
  for (int i = threadIdx.x; i < nb; i += kRedThreads) a += part[i];
  a = block_sum(a);
  if (threadIdx.x == 0) *out = a;
}
__global__ void k_kdif_refine(int n, double* x, const float* d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = x[i] + (double)d[i];
}
__global__ void k_kdif_update_T(DevMesh m, KdifState k) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  k.T[c] = k.T[c] + k.x[c] / k.cp;
}

// ---- fused conjugate gradients (single reduction per iteration) ----
// Chronopoulos and Gear's arrangement of Jacobi-preconditioned CG: with u = D^-1 r, w = S u,
// and p and s = S p carried by recurrences, both inner products of an iteration,
// gamma = r.u and delta = w.u, come from the same iterate, so an iteration is two launches
// and no host round trip:
//   A: x += alpha p, r -= alpha s, u = r / diag; gamma, r.r;   beta = gamma / gamma_old
//   B: w = S u, p = u + beta p, s = w + beta s; delta;         alpha = gamma / (delta - beta gamma / alpha_old)
// Each launch reduces in a fixed grid (block sums, then the last block to finish sums the
// block partials in block order): deterministic.  Scalars: scal[8] gamma, [9] alpha,
// [10] beta, [11] r.r, [12] delta.
constexpr int kFcgGamma = 8, kFcgAlpha = 9, kFcgBeta = 10, kFcgRR = 11, kFcgDelta = 12;

// the symmetrised matrix in difference form (kdif.hpp) and the Jacobi inverse
__global__ void __launch_bounds__(kBlock) k_kdif_ell(DevMesh m, KdifState k, double dt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t n = m.nci;
  double mc = m.cvol[c] / dt, d = mc;
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = k.cfo[sl * n + c];
    double a = 0.0;
    int nb = c;
    if (e >= 0) {
      const int f = e >> 1;
      if (f >= m.nfi) mc = mc - k.jac[f];
      else { a = -k.jac[f]; nb = k.cfon[sl * n + c]; }
      d = d - k.jac[f];
    }
    k.ell_a[sl * n + c] = a;
    k.ell_a32[sl * n + c] = (float)a;
    k.ell_nb[sl * n + c] = nb;
  }
  k.ell_m[c] = mc;
  k.dinv[c] = 1.0 / d;
}

// last block of a launch: true in every thread of the block that finished last
__device__ __forceinline__ bool kd_last_block(unsigned* count) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(count, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}
// sum of the block partials part[0..nb) in block order (every thread; valid in thread 0)
__device__ __forceinline__ double kd_sum_partials(const double* part, int nb) {
  double a = 0.0;
  for (int i = threadIdx.x; i < nb; i += kRedThreads) a += __ldcg(part + i);
  return block_sum(a);
}

// A (first = 1: start, x = 0, r = b; first = 2: restart from the current x and r)
__global__ void __launch_bounds__(kRedThreads) k_kdif_fcg_a(int n, KdifState k, int first) {
  const double alpha = first ? 0.0 : k.scal[kFcgAlpha];
  double g = 0.0, rr = 0.0;
  for (int i = blockIdx.x * kRedThreads + threadIdx.x; i < n; i += gridDim.x * kRedThreads) {
    double xi, ri;
    if (first == 1) { xi = 0.0; ri = k.bal[i]; }
    else if (first == 2) { xi = k.x[i]; ri = k.r[i]; }
    else { xi = k.x[i] + alpha * k.p[i]; ri = k.r[i] - alpha * k.s[i]; }
    const double ui = ri * k.dinv[i];
    k.x[i] = xi; k.r[i] = ri; k.z[i] = ui;
    g += ri * ui;
    rr += ri * ri;
  }
  g = block_sum(g);
  if (threadIdx.x == 0) k.part[blockIdx.x] = g;
  rr = block_sum(rr);
  if (threadIdx.x == 0) k.part[kRedBlocks + blockIdx.x] = rr;
  if (!kd_last_block(k.count)) return;
  const double gt = kd_sum_partials(k.part, gridDim.x);
  const double rt = kd_sum_partials(k.part + kRedBlocks, gridDim.x);
  if (threadIdx.x == 0) {
    k.scal[kFcgBeta] = first ? 0.0 : gt / k.scal[kFcgGamma];
    k.scal[kFcgGamma] = gt;
    k.scal[kFcgRR] = rt;
    if (first == 1) k.scal[3] = rt;   // |b|^2
    *k.count = 0u;
  }
}

// B: w = S u with FP64 (A32 = false) or FP32 (A32 = true) conductances
template <bool A32>
__global__ void __launch_bounds__(kRedThreads) k_kdif_fcg_b(int n, int ns, KdifState k, int first) {
  const double beta = k.scal[kFcgBeta];
  double dl = 0.0;
  for (int c = blockIdx.x * kRedThreads + threadIdx.x; c < n; c += gridDim.x * kRedThreads) {
    const double uc = k.z[c];
    double w = k.ell_m[c] * uc;
    for (int sl = 0; sl < ns; ++sl) {
      const double a = A32 ? (double)k.ell_a32[sl * (size_t)n + c] : k.ell_a[sl * (size_t)n + c];
      w = fma(a, uc - k.z[k.ell_nb[sl * (size_t)n + c]], w);
    }
    if (first) { k.p[c] = uc; k.s[c] = w; }
    else { k.p[c] = fma(beta, k.p[c], uc); k.s[c] = fma(beta, k.s[c], w); }
    dl += w * uc;
  }
  dl = block_sum(dl);
  if (threadIdx.x == 0) k.part[blockIdx.x] = dl;
  if (!kd_last_block(k.count + 1)) return;
  const double dt = kd_sum_partials(k.part, gridDim.x);
  if (threadIdx.x == 0) {
    const double gm = k.scal[kFcgGamma];
    k.scal[kFcgDelta] = dt;
    k.scal[kFcgAlpha] = first ? gm / dt : gm / (dt - beta * gm / k.scal[kFcgAlpha]);
    k.count[1] = 0u;
  }
}

// the true residual r = b - S x of the FP64 system, from which the iteration restarts when
// the operator changes from FP32 to FP64 conductances (continuing the old directions on the
// changed operator loses their conjugacy: on this stiff system the iteration stagnates)
__global__ void __launch_bounds__(kRedThreads) k_kdif_fcg_replace(int n, int ns, KdifState k) {
  for (int c = blockIdx.x * kRedThreads + threadIdx.x; c < n; c += gridDim.x * kRedThreads) {
    const double xc = k.x[c];
    double sx = k.ell_m[c] * xc;
    for (int sl = 0; sl < ns; ++sl)
      sx = fma(k.ell_a[sl * (size_t)n + c], xc - k.x[k.ell_nb[sl * (size_t)n + c]], sx);
    k.r[c] = k.bal[c] - sx;
  }
}

// ---- launchers ----
cudaError_t kdif_ell_build(const DevMesh& m, const KdifState& k, double dt, cudaStream_t st) {
  k_kdif_ell<<<nblk(m.nci), kBlock, 0, st>>>(m, k, dt);
  return cudaGetLastError();
}
cudaError_t kdif_fcg_a(const DevMesh& m, const KdifState& k, int first, cudaStream_t st) {
  k_kdif_fcg_a<<<red_grid(m.nci), kRedThreads, 0, st>>>(m.nci, k, first);
  return cudaGetLastError();
}
cudaError_t kdif_fcg_b(const DevMesh& m, const KdifState& k, int first, int f32, cudaStream_t st) {
  if (f32) k_kdif_fcg_b<true><<<red_grid(m.nci), kRedThreads, 0, st>>>(m.nci, m.nslot, k, first);
  else k_kdif_fcg_b<false><<<red_grid(m.nci), kRedThreads, 0, st>>>(m.nci, m.nslot, k, first);
  return cudaGetLastError();
}
cudaError_t kdif_fcg_replace(const DevMesh& m, const KdifState& k, cudaStream_t st) {
  k_kdif_fcg_replace<<<red_grid(m.nci), kRedThreads, 0, st>>>(m.nci, m.nslot, k);
  return cudaGetLastError();
}

cudaError_t kdif_residual(const DevMesh& m, const KdifState& k, double dt, cudaStream_t st) {
  if (m.ng > 0) k_kdif_ghost<<<nblk(m.ng), kBlock, 0, st>>>(m, k);
  if (k.scheme != TY_KDIF_COMPACT) k_kdif_grad<<<nblk(m.nci), kBlock, 0, st>>>(m, k);
  k_kdif_face<<<nblk(m.nf), kBlock, 0, st>>>(m, k);
  k_kdif_gather<<<nblk(m.nci), kBlock, 0, st>>>(m, k, dt, nullptr);
  return cudaGetLastError();
}
cudaError_t kdif_assemble(const DevMesh& m, const KdifState& k, double dt, int want32, cudaStream_t st) {
  k_kdif_diag<<<nblk(m.nci), kBlock, 0, st>>>(m, k, dt, want32);
  if (want32) k_kdif_jac32<<<std::min<unsigned>(nblk(m.nf), 4 * kRedBlocks), kBlock, 0, st>>>(k, m.nf);
  return cudaGetLastError();
}
cudaError_t kdif_matvec(const DevMesh& m, const KdifState& k, const double* x, double* y, cudaStream_t st) {
  k_kdif_mv<double><<<red_grid(m.nci), kRedThreads, 0, st>>>(m, k, x, y, k.diag, k.jac, nullptr);
  return cudaGetLastError();
}
// CG on S x = r (FP64: r = bal; FP32: r32 = refinement residual), scalars in k.scal
cudaError_t kdif_cg_start(const DevMesh& m, const KdifState& k, int f32, cudaStream_t st) {
  const unsigned g = red_grid(m.nci);
  if (f32) k_kdif_cg0<float><<<g, kRedThreads, 0, st>>>(m.nci, k.x32, k.r32, k.z32, k.p32, k.diag32, k.part);
  else {
    cudaMemcpyAsync(k.r, k.bal, m.nci * sizeof(double), cudaMemcpyDeviceToDevice, st);
    k_kdif_cg0<double><<<g, kRedThreads, 0, st>>>(m.nci, k.x, k.r, k.z, k.p, k.diag, k.part);
  }
  k_kdif_final<<<1, kRedThreads, 0, st>>>(k.part, (int)g, 0, k.scal);
  return cudaGetLastError();
}
cudaError_t kdif_cg_iter(const DevMesh& m, const KdifState& k, int f32, cudaStream_t st) {
  const unsigned g = red_grid(m.nci);
  const unsigned g2 = std::min<unsigned>(nblk(m.nci), 4 * kRedBlocks);
  if (f32) {
    k_kdif_mv<float><<<g, kRedThreads, 0, st>>>(m, k, k.p32, k.q32, k.diag32, k.jac32, k.part);
    k_kdif_final<<<1, kRedThreads, 0, st>>>(k.part, (int)g, 1, k.scal);
    k_kdif_cg1<float><<<g, kRedThreads, 0, st>>>(m.nci, k.x32, k.r32, k.z32, k.p32, k.q32, k.diag32, k.scal, k.part);
    k_kdif_final<<<1, kRedThreads, 0, st>>>(k.part, (int)g, 2, k.scal);
    k_kdif_cg2<float><<<g2, kBlock, 0, st>>>(m.nci, k.z32, k.p32, k.scal);
  } else {
    k_kdif_mv<double><<<g, kRedThreads, 0, st>>>(m, k, k.p, k.q, k.diag, k.jac, k.part);
    k_kdif_final<<<1, kRedThreads, 0, st>>>(k.part, (int)g, 1, k.scal);
    k_kdif_cg1<double><<<g, kRedThreads, 0, st>>>(m.nci, k.x, k.r, k.z, k.p, k.q, k.diag, k.scal, k.part);
    k_kdif_final<<<1, kRedThreads, 0, st>>>(k.part, (int)g, 2, k.scal);
    k_kdif_cg2<double><<<g2, kBlock, 0, st>>>(m.nci, k.z, k.p, k.scal);
  }
  k_kdif_shift<<<1, 1, 0, st>>>(k.scal);
  return cudaGetLastError();
}
cudaError_t kdif_residual64(const DevMesh& m, const KdifState& k, cudaStream_t st) {
  const unsigned g = red_grid(m.nci);
  k_kdif_res64<<<g, kRedThreads, 0, st>>>(m, k, k.part);
  k_kdif_final1<<<1, kRedThreads, 0, st>>>(k.part, (int)g, k.scal + 5);
  return cudaGetLastError();
}
cudaError_t kdif_refine(const DevMesh& m, const KdifState& k, cudaStream_t st) {
  k_kdif_refine<<<std::min<unsigned>(nblk(m.nci), 4 * kRedBlocks), kBlock, 0, st>>>(m.nci, k.x, k.x32);
  return cudaGetLastError();
}
cudaError_t kdif_update_T(const DevMesh& m, const KdifState& k, cudaStream_t st) {
  k_kdif_update_T<<<nblk(m.nci), kBlock, 0, st>>>(m, k);
  return cudaGetLastError();
}

}  // namespace TY_KNS
}  // namespace tyk
