// Adjoint (vector-Jacobian product) of the first-order residual, instantiated per mode after
// kernels.cuh.  New: Typhon has no adjoint (its inverse mode differentiates by finite
// differences, SOURCE/MAIN/inverse_calc_sensi.f90).
//
// R_c = dt/V_c sum_f (+-) F_f(U) S_f with face states Q_L = prim(U_fc1), Q_R = prim(U_fc2) or
// the boundary state built from Q_L (periodic: the partner's inside cell).  Given lambda_R,
//   lambda_F(f) = S_f (dt/V_fc2 lambda_R(fc2) [interior faces] - dt/V_fc1 lambda_R(fc1)),
//   lambda_U   += (dF/dU_L)^T lambda_F on fc1 and (dF/dU_R)^T lambda_F on the right cell,
// the face loop reversed into a gather: a face kernel writes both products, a cell kernel
// sums a cell's faces (and, for a periodic boundary face, the product of its partner face,
// whose right state is this cell).  dF/dU comes from forward-mode dual numbers through the
// same flux formulas as the exact-mode residual (cons -> prim, boundary state, flux), one
// sweep for the 5 left and one for the 5 right directions.
#pragma once
#include "adjoint.hpp"

namespace tyk {
namespace TY_KNS {

template <int N>
struct Dual {
  double v;
  double d[N];
  __device__ Dual() {}
  __device__ Dual(double x) : v(x) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
};
#define TY_DUAL_BIN(op, dexpr)                                                                       \
  template <int N>                                                                                   \
  __device__ __forceinline__ Dual<N> operator op(const Dual<N>& a, const Dual<N>& b) {               \
    Dual<N> r;                                                                                       \
    r.v = a.v op b.v;                                                                                \
    _Pragma("unroll") for (int i = 0; i < N; ++i) r.d[i] = dexpr;                                    \
    return r;                                                                                        \
  }
TY_DUAL_BIN(+, a.d[i] + b.d[i])
TY_DUAL_BIN(-, a.d[i] - b.d[i])
TY_DUAL_BIN(*, a.d[i] * b.v + a.v * b.d[i])
#undef TY_DUAL_BIN
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> __device__ __forceinline__ Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> __device__ __forceinline__ Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> __device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N> __device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N> __device__ __forceinline__ Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) { return a * -1.0; }
template <int N> __device__ __forceinline__ Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = ::sqrt(a.v);
  const double h = 0.5 / r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * h;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> fabs(const Dual<N>& a) { return signbit(a.v) ? -a : a; }
template <int N> __device__ __forceinline__ Dual<N> fmin(const Dual<N>& a, const Dual<N>& b) { return b.v < a.v ? b : a; }
template <int N> __device__ __forceinline__ Dual<N> fmax(const Dual<N>& a, const Dual<N>& b) { return b.v > a.v ? b : a; }
template <int N> __device__ __forceinline__ double val(const Dual<N>& a) { return a.v; }
__device__ __forceinline__ double val(double a) { return a; }

// cons -> prim (calc_varprim_ns.f90), exact-mode operation order
template <class T>
__device__ void prim_t(double g, const T* c, T* q) {
  T rho = c[0];
  T vx = c[2] / rho, vy = c[3] / rho, vz = c[4] / rho;
  T ec = 0.5 * rho * (vx * vx + vy * vy + vz * vz);
  q[0] = rho;
  q[1] = (g - 1.0) * (c[1] - ec);
  q[2] = vx; q[3] = vy; q[4] = vz;
}

template <class T>
__device__ void flux_rusanov_t(double g, const T* L, const T* R, double nx, double ny, double nz, T* F) {
  const double ig1 = 1.0 / (g - 1.0);
  T vnl = L[2] * nx + L[3] * ny + L[4] * nz;
  T vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  T al = sqrt(g * L[1] / L[0]);
  T ar = sqrt(g * R[1] / R[0]);
  T ray = fmax(fabs(vnl) + al, fabs(vnr) + ar);
  T rel = ig1 * L[1] + 0.5 * L[0] * (L[2] * L[2] + L[3] * L[3] + L[4] * L[4]);
  T rer = ig1 * R[1] + 0.5 * R[0] * (R[2] * R[2] + R[3] * R[3] + R[4] * R[4]);
  F[0] = 0.5 * ((vnl + ray) * L[0] + (vnr - ray) * R[0]);
  F[1] = 0.5 * ((vnl + ray) * rel + (vnr - ray) * rer + vnl * L[1] + vnr * R[1]);
  T a = (vnl + ray) * L[0], b = (vnr - ray) * R[0], pp = L[1] + R[1];
  F[2] = 0.5 * ((a * L[2] + b * R[2]) + pp * nx);
  F[3] = 0.5 * ((a * L[3] + b * R[3]) + pp * ny);
  F[4] = 0.5 * ((a * L[4] + b * R[4]) + pp * nz);
}

template <class T>
__device__ void flux_hllc_t(double g, const T* L, const T* R, double nx, double ny, double nz, T* F) {
  const double ig1 = 1.0 / (g - 1.0), gig1 = g / (g - 1.0);
  T t1 = sqrt(R[0] / L[0]);
  T roe_rho = L[0] * t1;
  T kl = 1.0 / (1.0 + t1);
  T kr = t1 * kl;
  T rux = kl * L[2] + kr * R[2], ruy = kl * L[3] + kr * R[3], ruz = kl * L[4] + kr * R[4];
  T sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4];
  T sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  T h1 = gig1 * L[1] / L[0] + 0.5 * sqL;
  T h2 = gig1 * R[1] / R[0] + 0.5 * sqR;
  h1 = kl * h1 + kr * h2;
  T roe_p = (h1 - 0.5 * (rux * rux + ruy * ruy + ruz * ruz)) * roe_rho / gig1;
  T vnl = L[2] * nx + L[3] * ny + L[4] * nz;
  T vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  T al = sqrt(g * L[1] / L[0]);
  T ar = sqrt(g * R[1] / R[0]);
  T vm = rux * nx + ruy * ny + ruz * nz;
  T am = sqrt(g * roe_p / roe_rho);
  T rel = ig1 * L[1] + 0.5 * L[0] * sqL;
  T rer = ig1 * R[1] + 0.5 * R[0] * sqR;
  T sl = fmin(vnl - al, vm - am);
  T sr = fmax(vnr + ar, vm + am);
  if (val(sl) >= 0.0) {
    T m0 = vnl * L[0];
    F[0] = m0;
    F[1] = vnl * (rel + L[1]);
    F[2] = m0 * L[2] + L[1] * nx; F[3] = m0 * L[3] + L[1] * ny; F[4] = m0 * L[4] + L[1] * nz;
  } else if (val(sr) <= 0.0) {
    T m0 = vnr * R[0];
    F[0] = m0;
    F[1] = vnr * (rer + R[1]);
    F[2] = m0 * R[2] + R[1] * nx; F[3] = m0 * R[3] + R[1] * ny; F[4] = m0 * R[4] + R[1] * nz;
  } else {
    T rqL = L[0] * (sl - vnl);
    T rqR = R[0] * (sr - vnr);
    T Sst = (rqR * vnr - rqL * vnl - R[1] + L[1]) / (rqR - rqL);
    const bool left = val(Sst) >= 0.0;
    const T* Q = left ? L : R;
    T s = left ? sl : sr, vq = left ? vnl : vnr, rq = left ? rqL : rqR, re = left ? rel : rer;
    T iks = 1.0 / (s - Sst);
    T rst = rq * iks;
    T pst = Q[1] - rq * (vq - Sst);
    T dp = pst - Q[1];
    T rvx = iks * ((rq * Q[2]) + dp * nx), rvy = iks * ((rq * Q[3]) + dp * ny), rvz = iks * ((rq * Q[4]) + dp * nz);
    T rest = iks * (re * (s - vq) - Q[1] * vq + pst * Sst);
    F[0] = Sst * rst;
    F[1] = Sst * (rest + pst);
    F[2] = (Sst * rvx) + (pst * nx); F[3] = (Sst * rvy) + (pst * ny); F[4] = (Sst * rvz) + (pst * nz);
  }
}

template <class T>
__device__ void flux_roe_t(double g, double eps, const T* L, const T* R, double nx, double ny, double nz, T* F) {
  const double ig1 = 1.0 / (g - 1.0), gig1 = g / (g - 1.0);
  T t1 = sqrt(R[0] / L[0]);
  T rroe = L[0] * t1;
  T kl = 1.0 / (1.0 + t1), kr = t1 * kl;
  T ux = kl * L[2] + kr * R[2], uy = kl * L[3] + kr * R[3], uz = kl * L[4] + kr * R[4];
  T sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4];
  T sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  T hl = gig1 * L[1] / L[0] + 0.5 * sqL;
  T hr = gig1 * R[1] / R[0] + 0.5 * sqR;
  T hroe = kl * hl + kr * hr;
  T q2 = ux * ux + uy * uy + uz * uz;
  T a2 = (g - 1.0) * (hroe - 0.5 * q2);
  T a = sqrt(a2);
  T vn = ux * nx + uy * ny + uz * nz;
  T vnl = L[2] * nx + L[3] * ny + L[4] * nz;
  T vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  T rel = ig1 * L[1] + 0.5 * L[0] * sqL;
  T rer = ig1 * R[1] + 0.5 * R[0] * sqR;
  T drho = R[0] - L[0], dp = R[1] - L[1], dvn = vnr - vnl;
  T dux = R[2] - L[2], duy = R[3] - L[3], duz = R[4] - L[4];
  T al1 = (dp - rroe * a * dvn) / (2.0 * a2);
  T al5 = (dp + rroe * a * dvn) / (2.0 * a2);
  T al2 = drho - dp / a2;
  T dutx = dux - dvn * nx, duty = duy - dvn * ny, dutz = duz - dvn * nz;
  T l1 = fabs(vn - a), l5 = fabs(vn + a), l2 = fabs(vn);
  T delta = eps * a;
  if (val(l1) < val(delta)) l1 = (l1 * l1 + delta * delta) / (2.0 * delta);
  if (val(l5) < val(delta)) l5 = (l5 * l5 + delta * delta) / (2.0 * delta);
  T w1 = l1 * al1, w2 = l2 * al2, w5 = l5 * al5, ws = l2 * rroe;
  T d_mass = w1 + w2 + w5;
  T dmx = w1 * (ux - a * nx) + w2 * ux + w5 * (ux + a * nx) + ws * dutx;
  T dmy = w1 * (uy - a * ny) + w2 * uy + w5 * (uy + a * ny) + ws * duty;
  T dmz = w1 * (uz - a * nz) + w2 * uz + w5 * (uz + a * nz) + ws * dutz;
  T d_ener = w1 * (hroe - a * vn) + w2 * (0.5 * q2) + w5 * (hroe + a * vn) +
             ws * ((ux * dux + uy * duy + uz * duz) - vn * dvn);
  T ml = vnl * L[0], mr = vnr * R[0];
  F[0] = 0.5 * (ml + mr - d_mass);
  F[1] = 0.5 * (vnl * (rel + L[1]) + vnr * (rer + R[1]) - d_ener);
  F[2] = 0.5 * ((ml * L[2] + L[1] * nx) + (mr * R[2] + R[1] * nx) - dmx);
  F[3] = 0.5 * ((ml * L[3] + L[1] * ny) + (mr * R[3] + R[1] * ny) - dmy);
  F[4] = 0.5 * ((ml * L[4] + L[1] * nz) + (mr * R[4] + R[1] * nz) - dmz);
}

// right state of a boundary face built from the left one (first order)
template <class T>
__device__ void bc_state_t(const DevMesh& m, const SpatOpts& o, int f, int kind, const T* QL, T* QR) {
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  if (kind == TY_BC_SYMMETRY) {
    T dn = 2.0 * (QL[2] * nx + QL[3] * ny + QL[4] * nz);
    QR[0] = QL[0]; QR[1] = QL[1];
    QR[2] = QL[2] - dn * nx; QR[3] = QL[3] - dn * ny; QR[4] = QL[4] - dn * nz;
  } else if (kind == TY_BC_WALL || kind == TY_BC_NOSLIP) {
    QR[0] = kind == TY_BC_NOSLIP ? QL[0] : QL[1];
    QR[1] = QL[1];
    QR[2] = 2.0 * d3(m.fwall, m.ldf, f, 0) - QL[2];
    QR[3] = 2.0 * d3(m.fwall, m.ldf, f, 1) - QL[3];
    QR[4] = 2.0 * d3(m.fwall, m.ldf, f, 2) - QL[4];
  } else {  // far field, kind fixed by the free stream
    const double* qi = o.farfield;
    const double vn = qi[2] * nx + qi[3] * ny + qi[4] * nz;
    const double c = ::sqrt(o.gamma * qi[1] / qi[0]);
    if (vn <= -c) {
#pragma unroll
      for (int v = 0; v < 5; ++v) QR[v] = T(qi[v]);
    } else if (vn < -1e-8 * c) {
      QR[0] = T(qi[0]); QR[1] = QL[1]; QR[2] = T(qi[2]); QR[3] = T(qi[3]); QR[4] = T(qi[4]);
    } else if (vn < c) {
      QR[0] = QL[0]; QR[1] = T(qi[1]); QR[2] = QL[2]; QR[3] = QL[3]; QR[4] = QL[4];
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) QR[v] = QL[v];
    }
  }
}

template <int SCH, class T>
__device__ void face_flux_t(const DevMesh& m, const SpatOpts& o, int f, const T* UL, const T* UR, T* F) {
  T QL[5], QR[5];
  prim_t(o.gamma, UL, QL);
  const int kind = f < m.nfi ? TY_BC_INTERIOR : m.fbc[f];
  if (kind == TY_BC_INTERIOR || kind == TY_BC_PERIODIC) prim_t(o.gamma, UR, QR);
  else bc_state_t(m, o, f, kind, QL, QR);
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  if constexpr (SCH == TY_SCH_HLLC) flux_hllc_t(o.gamma, QL, QR, nx, ny, nz, F);
  else if constexpr (SCH == TY_SCH_RUSANOV) flux_rusanov_t(o.gamma, QL, QR, nx, ny, nz, F);
  else flux_roe_t(o.gamma, o.entropy_fix, QL, QR, nx, ny, nz, F);
}

// per face: lambda_F, then (dF/dU_L)^T lambda_F and (dF/dU_R)^T lambda_F into lam_face [10][ldf]
template <int SCH>
__global__ void __launch_bounds__(128) k_adj_face(DevMesh m, SpatOpts o, const double* __restrict__ u,
                                                  const double* __restrict__ lamR, double dt,
                                                  double* __restrict__ lam_face) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const size_t ld = m.ldc, lf = m.ldf;
  const int c1 = m.fc1[f];
  const int kind = f < m.nfi ? TY_BC_INTERIOR : m.fbc[f];
  const int cr = kind == TY_BC_INTERIOR ? m.fc2[f] : (kind == TY_BC_PERIODIC ? m.fc1[m.part[f]] : c1);
  const double S = m.fs[f];
  double lF[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double a = -(dt / m.cvol[c1]) * lamR[v * ld + c1];
    if (kind == TY_BC_INTERIOR) a = a + (dt / m.cvol[cr]) * lamR[v * ld + cr];
    lF[v] = S * a;
  }
  double uL[5], uR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) { uL[v] = u[v * ld + c1]; uR[v] = u[v * ld + cr]; }
  const int nside = (kind == TY_BC_INTERIOR || kind == TY_BC_PERIODIC) ? 2 : 1;
#pragma unroll 1
  for (int side = 0; side < 2; ++side) {
    if (side >= nside) {  // the right state is built from the left one: no right product
#pragma unroll
      for (int j = 0; j < 5; ++j) lam_face[(5 + j) * lf + f] = 0.0;
      break;
    }
    Dual<5> UL[5], UR[5], F[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      UL[v] = Dual<5>(uL[v]);
      UR[v] = Dual<5>(uR[v]);
      if (side == 0) UL[v].d[v] = 1.0;
      else UR[v].d[v] = 1.0;
    }
    face_flux_t<SCH>(m, o, f, UL, UR, F);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      double s = 0.0;
#pragma unroll
      for (int v = 0; v < 5; ++v) s += lF[v] * F[v].d[j];
      lam_face[(5 * side + j) * lf + f] = s;
    }
  }
}

__global__ void __launch_bounds__(kBlock) k_adj_cell(DevMesh m, const double* __restrict__ lam_face,
                                                     double* __restrict__ lamU) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t lf = m.ldf;
  double s[5] = {0, 0, 0, 0, 0};
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = m.cf[sl * (size_t)m.nci + c];
    if (e < 0) break;
    const int f = e >> 1, side = e & 1;
#pragma unroll
    for (int v = 0; v < 5; ++v) s[v] += lam_face[(5 * side + v) * lf + f];
    if (!side && f >= m.nfi && m.fbc[f] == TY_BC_PERIODIC) {
      const int p = m.part[f];  // the partner face's right state is this cell
#pragma unroll
      for (int v = 0; v < 5; ++v) s[v] += lam_face[(5 + v) * lf + p];
    }
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) lamU[v * (size_t)m.ldc + c] = s[v];
}

cudaError_t adjoint_vjp(const DevMesh& m, const SpatOpts& o, const double* u, const double* lamR, double dt,
                        double* lam_face, double* lamU, cudaStream_t st) {
  const unsigned gf = (unsigned)((m.nf + 127) / 128);
  if (o.scheme == TY_SCH_HLLC) k_adj_face<TY_SCH_HLLC><<<gf, 128, 0, st>>>(m, o, u, lamR, dt, lam_face);
  else if (o.scheme == TY_SCH_RUSANOV) k_adj_face<TY_SCH_RUSANOV><<<gf, 128, 0, st>>>(m, o, u, lamR, dt, lam_face);
  else k_adj_face<TY_SCH_ROE><<<gf, 128, 0, st>>>(m, o, u, lamR, dt, lam_face);
  k_adj_cell<<<nblk(m.nci), kBlock, 0, st>>>(m, lam_face, lamU);
  return cudaGetLastError();
}

}  // namespace TY_KNS
}  // namespace tyk
