// Face fluxes of the first-order residual as templates over the number type (double, or
// forward-mode dual numbers), and their reverse-mode derivatives written by hand.  Host and
// device code: the dual-number forms are the cross-check of the hand-written ones.
//
// Operation order follows the exact-mode residual kernels (calc_varprim_ns.f90 for cons ->
// prim; SOURCE/VALE/calc_flux_rusanov.f90, calc_flux_hllc.f90, calc_flux_roe.f90 for the
// fluxes), so that the primal recomputed here equals the residual's.  The reverse forms take
// Fb = lambda_F and add (dF/dL)^T Fb and (dF/dR)^T Fb to Lb and Rb (L, R primitive states
// rho, p, u, v, w; n the unit face normal).
#pragma once
#include <cmath>

// The fast-mode kernels (TY_FAST) take the Newton-Raphson reciprocal and square root of
// fastmath.cuh in the reverse forms; the exact mode and the host take IEEE division and
// square root.
#if defined(TY_FAST) && TY_FAST && defined(__CUDACC__)
#include "fastmath.cuh"
#define TY_AD_NR 1
#else
#define TY_AD_NR 0
#endif

#ifdef __CUDACC__
#define TY_AD __host__ __device__ __forceinline__
#else
#define TY_AD inline
#endif

namespace tyk {
namespace adflux {

using std::signbit;

template <int N>
struct Dual {
  double v;
  double d[N];
  TY_AD Dual() {}
  TY_AD Dual(double x) : v(x) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
};
#define TY_DUAL_BIN(op, dexpr)                                                                       \
  template <int N>                                                                                   \
  TY_AD Dual<N> operator op(const Dual<N>& a, const Dual<N>& b) {               \
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
TY_AD Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N> TY_AD Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> TY_AD Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> TY_AD Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> TY_AD Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> TY_AD Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N> TY_AD Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N> TY_AD Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N> TY_AD Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> TY_AD Dual<N> operator-(const Dual<N>& a) { return a * -1.0; }
template <int N> TY_AD Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = ::sqrt(a.v);
  const double h = 0.5 / r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * h;
  return r;
}
template <int N> TY_AD Dual<N> fabs(const Dual<N>& a) { return signbit(a.v) ? -a : a; }
template <int N> TY_AD Dual<N> fmin(const Dual<N>& a, const Dual<N>& b) { return b.v < a.v ? b : a; }
template <int N> TY_AD Dual<N> fmax(const Dual<N>& a, const Dual<N>& b) { return b.v > a.v ? b : a; }
template <int N> TY_AD double val(const Dual<N>& a) { return a.v; }
TY_AD double val(double a) { return a; }

// cons -> prim (calc_varprim_ns.f90), exact-mode operation order
template <class T>
TY_AD void prim_t(double g, const T* c, T* q) {
  T rho = c[0];
  T vx = c[2] / rho, vy = c[3] / rho, vz = c[4] / rho;
  T ec = 0.5 * rho * (vx * vx + vy * vy + vz * vz);
  q[0] = rho;
  q[1] = (g - 1.0) * (c[1] - ec);
  q[2] = vx; q[3] = vy; q[4] = vz;
}

template <class T>
TY_AD void flux_rusanov_t(double g, const T* L, const T* R, double nx, double ny, double nz, T* F) {
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
TY_AD void flux_hllc_t(double g, const T* L, const T* R, double nx, double ny, double nz, T* F) {
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
TY_AD void flux_roe_t(double g, double eps, const T* L, const T* R, double nx, double ny, double nz, T* F) {
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

// The reverse forms below recompute the forward quantities they need with reciprocals
// (1/rho, 1/a, ...) in place of the forward formulas' divisions: derivative values agree
// with the dual-number forms to rounding, at a fraction of the FP64 divide/square-root work.  ad_rcp, ad_div and ad_sqrt are IEEE
// operations except in the fast-mode kernels (Newton-Raphson, within a few ulp).

TY_AD double ad_rcp(double a) {
#if TY_AD_NR && defined(__CUDA_ARCH__)
  return rcp_nr(a);
#else
  return 1.0 / a;
#endif
}
TY_AD double ad_div(double a, double b) {
#if TY_AD_NR && defined(__CUDA_ARCH__)
  return a * rcp_nr(b);
#else
  return a / b;
#endif
}
TY_AD double ad_sqrt(double a) {
#if TY_AD_NR && defined(__CUDA_ARCH__)
  return sqrt_nr(a);
#else
  return ::sqrt(a);
#endif
}

// cons -> prim with the reciprocal of the density; returns 1/rho
TY_AD double prim_r(double g, const double* c, double* q) {
  const double ir = ad_rcp(c[0]);
  const double vx = c[2] * ir, vy = c[3] * ir, vz = c[4] * ir;
  q[0] = c[0];
  q[1] = (g - 1.0) * (c[1] - 0.5 * c[0] * (vx * vx + vy * vy + vz * vz));
  q[2] = vx; q[3] = vy; q[4] = vz;
  return ir;
}

// reverse of cons -> prim: Ub += (dq/dU)^T qb at the conservative state U (ir = 1/rho)
TY_AD void prim_vjp(double g, const double* U, double ir, const double* qb, double* Ub) {
  const double u[3] = {U[2] * ir, U[3] * ir, U[4] * ir};
  const double u2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double ecb = -qb[1] * (g - 1.0);  // adjoint of the kinetic energy 0.5 rho |u|^2
  Ub[1] += qb[1] * (g - 1.0);
  double r0 = qb[0] + ecb * 0.5 * u2;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double ubk = (qb[2 + k] + ecb * U[0] * u[k]) * ir;  // adjoint of u_k, over rho
    Ub[2 + k] += ubk;
    r0 -= ubk * u[k];
  }
  Ub[0] += r0;
}

// Reverse of flux_roe_t: Lb += (dF/dL)^T Fb, Rb += (dF/dR)^T Fb, L and R primitive.
TY_AD void roe_vjp(double g, double eps, const double* L, const double* R, double nx, double ny, double nz,
                   const double* Fb, double* Lb, double* Rb) {
  const double n[3] = {nx, ny, nz};
  const double g1 = g - 1.0, ig1 = ad_rcp(g1), gig1 = g * ig1;
  const double iL = ad_rcp(L[0]), iR = ad_rcp(R[0]);
  // forward
  const double t1 = ad_sqrt(R[0] * iL), it1 = t1 * L[0] * iR;
  const double rroe = L[0] * t1;
  const double kl = ad_rcp(1.0 + t1), kr = t1 * kl;
  double u[3], du[3], dut[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = kl * L[2 + k] + kr * R[2 + k];
  const double sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4];
  const double sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  const double hl = gig1 * L[1] * iL + 0.5 * sqL, hr = gig1 * R[1] * iR + 0.5 * sqR;
  const double hroe = kl * hl + kr * hr;
  const double q2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double a2 = g1 * (hroe - 0.5 * q2);
  const double a = ad_sqrt(a2), ia = ad_rcp(a), ia2 = ia * ia;
  const double vn = u[0] * nx + u[1] * ny + u[2] * nz;
  const double vnl = L[2] * nx + L[3] * ny + L[4] * nz, vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  const double rel = ig1 * L[1] + 0.5 * L[0] * sqL, rer = ig1 * R[1] + 0.5 * R[0] * sqR;
  const double dp = R[1] - L[1], dvn = vnr - vnl, drho = R[0] - L[0];
#pragma unroll
  for (int k = 0; k < 3; ++k) { du[k] = R[2 + k] - L[2 + k]; dut[k] = du[k] - dvn * n[k]; }
  const double al1 = (dp - rroe * a * dvn) * (0.5 * ia2);
  const double al5 = (dp + rroe * a * dvn) * (0.5 * ia2);
  const double al2 = drho - dp * ia2;
  const double l1o = ::fabs(vn - a), l5o = ::fabs(vn + a), l2 = ::fabs(vn);
  const double delta = eps * a;
  const bool fix1 = l1o < delta, fix5 = l5o < delta;
  const double idl = (fix1 || fix5) ? ad_rcp(delta) : 0.0;
  const double l1 = fix1 ? (l1o * l1o + delta * delta) * (0.5 * idl) : l1o;
  const double l5 = fix5 ? (l5o * l5o + delta * delta) * (0.5 * idl) : l5o;
  const double w1 = l1 * al1, w2 = l2 * al2, w5 = l5 * al5, ws = l2 * rroe;
  const double udu = u[0] * du[0] + u[1] * du[1] + u[2] * du[2];
  const double ml = vnl * L[0], mr = vnr * R[0];
  // reverse
  double mlb = 0.5 * Fb[0], mrb = 0.5 * Fb[0];
  double dmb[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    mlb += 0.5 * Fb[2 + k] * L[2 + k];
    mrb += 0.5 * Fb[2 + k] * R[2 + k];
    Lb[2 + k] += 0.5 * Fb[2 + k] * ml;
    Rb[2 + k] += 0.5 * Fb[2 + k] * mr;
    Lb[1] += 0.5 * Fb[2 + k] * n[k];
    Rb[1] += 0.5 * Fb[2 + k] * n[k];
    dmb[k] = -0.5 * Fb[2 + k];
  }
  const double d_massb = -0.5 * Fb[0];
  double vnlb = 0.5 * Fb[1] * (rel + L[1]), vnrb = 0.5 * Fb[1] * (rer + R[1]);
  const double relb = 0.5 * Fb[1] * vnl, rerb = 0.5 * Fb[1] * vnr;
  Lb[1] += 0.5 * Fb[1] * vnl;
  Rb[1] += 0.5 * Fb[1] * vnr;
  const double enb = -0.5 * Fb[1];
  vnlb += mlb * L[0]; Lb[0] += mlb * vnl;
  vnrb += mrb * R[0]; Rb[0] += mrb * vnr;
  double w1b = enb * (hroe - a * vn) + d_massb, w2b = enb * (0.5 * q2) + d_massb;
  double w5b = enb * (hroe + a * vn) + d_massb, wsb = enb * (udu - vn * dvn);
  double hroeb = enb * (w1 + w5);
  double ab = enb * (w5 - w1) * vn;
  double vnb = enb * ((w5 - w1) * a - ws * dvn);
  double q2b = enb * 0.5 * w2;
  double dvnb = -enb * ws * vn;
  double ub[3], dub[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    ub[k] = enb * ws * du[k] + dmb[k] * (w1 + w2 + w5);
    dub[k] = enb * ws * u[k];
    w1b += dmb[k] * (u[k] - a * n[k]);
    w2b += dmb[k] * u[k];
    w5b += dmb[k] * (u[k] + a * n[k]);
    wsb += dmb[k] * dut[k];
    ab += dmb[k] * (w5 - w1) * n[k];
    const double dutb = dmb[k] * ws;
    dub[k] += dutb;
    dvnb -= dutb * n[k];
  }
  const double l1b = w1b * al1, al1b = w1b * l1, l2b = w2b * al2 + wsb * rroe, al2b = w2b * l2;
  const double l5b = w5b * al5, al5b = w5b * l5;
  double rroeb = wsb * l2;
  double deltab = 0.0, l1ob = l1b, l5ob = l5b;
  if (fix1) { l1ob = l1b * l1o * idl; deltab += l1b * (delta * delta - l1o * l1o) * (0.5 * idl * idl); }
  if (fix5) { l5ob = l5b * l5o * idl; deltab += l5b * (delta * delta - l5o * l5o) * (0.5 * idl * idl); }
  ab += eps * deltab;
  const double s1 = signbit(vn - a) ? -1.0 : 1.0, s5 = signbit(vn + a) ? -1.0 : 1.0, s2 = signbit(vn) ? -1.0 : 1.0;
  vnb += l1ob * s1 + l5ob * s5 + l2b * s2;
  ab += l5ob * s5 - l1ob * s1;
  const double drhob = al2b;
  double dpb = -al2b * ia2, a2b = al2b * dp * ia2 * ia2;
  const double N5b = al5b * (0.5 * ia2), N1b = al1b * (0.5 * ia2);
  a2b -= (al5b * al5 + al1b * al1) * ia2;
  dpb += N5b + N1b;
  rroeb += (N5b - N1b) * a * dvn;
  ab += (N5b - N1b) * rroe * dvn;
  dvnb += (N5b - N1b) * rroe * a;
#pragma unroll
  for (int k = 0; k < 3; ++k) { Rb[2 + k] += dub[k]; Lb[2 + k] -= dub[k]; }
  Rb[0] += drhob; Lb[0] -= drhob;
  Rb[1] += dpb; Lb[1] -= dpb;
  vnrb += dvnb; vnlb -= dvnb;
  Lb[1] += relb * ig1; Lb[0] += relb * 0.5 * sqL;
  Rb[1] += rerb * ig1; Rb[0] += rerb * 0.5 * sqR;
  double sqLb = relb * 0.5 * L[0], sqRb = rerb * 0.5 * R[0];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    Lb[2 + k] += vnlb * n[k];
    Rb[2 + k] += vnrb * n[k];
    ub[k] += vnb * n[k];
  }
  a2b += ab * 0.5 * ia;
  hroeb += a2b * g1;
  q2b -= a2b * g1 * 0.5;
#pragma unroll
  for (int k = 0; k < 3; ++k) ub[k] += q2b * 2.0 * u[k];
  double klb = hroeb * hl, krb = hroeb * hr;
  const double hlb = hroeb * kl, hrb = hroeb * kr;
  Lb[1] += hlb * gig1 * iL; Lb[0] -= hlb * gig1 * L[1] * iL * iL; sqLb += hlb * 0.5;
  Rb[1] += hrb * gig1 * iR; Rb[0] -= hrb * gig1 * R[1] * iR * iR; sqRb += hrb * 0.5;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    Lb[2 + k] += sqLb * 2.0 * L[2 + k] + ub[k] * kl;
    Rb[2 + k] += sqRb * 2.0 * R[2 + k] + ub[k] * kr;
    klb += ub[k] * L[2 + k];
    krb += ub[k] * R[2 + k];
  }
  double t1b = krb * kl;
  klb += krb * t1;
  t1b -= klb * kl * kl;
  Lb[0] += rroeb * t1;
  t1b += rroeb * L[0];
  const double rb = t1b * 0.5 * it1;  // t1 = sqrt(R0 / L0)
  Rb[0] += rb * iL;
  Lb[0] -= rb * R[0] * iL * iL;
}

// Reverse of flux_rusanov_t.
TY_AD void rusanov_vjp(double g, const double* L, const double* R, double nx, double ny, double nz,
                       const double* Fb, double* Lb, double* Rb) {
  const double n[3] = {nx, ny, nz};
  const double ig1 = ad_rcp(g - 1.0);
  const double iL = ad_rcp(L[0]), iR = ad_rcp(R[0]);
  const double vnl = L[2] * nx + L[3] * ny + L[4] * nz, vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  const double al = ad_sqrt(g * L[1] * iL), ar = ad_sqrt(g * R[1] * iR);
  const double cl = ::fabs(vnl) + al, cr = ::fabs(vnr) + ar;
  const bool right = cr > cl;
  const double ray = right ? cr : cl;
  const double sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4], sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  const double rel = ig1 * L[1] + 0.5 * L[0] * sqL, rer = ig1 * R[1] + 0.5 * R[0] * sqR;
  const double sl = vnl + ray, sr = vnr - ray;
  const double A = sl * L[0], B = sr * R[0];
  double ppb = 0.0, Ab = 0.0, Bb = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double fb = 0.5 * Fb[2 + k];
    ppb += fb * n[k];
    Ab += fb * L[2 + k];
    Bb += fb * R[2 + k];
    Lb[2 + k] += fb * A;
    Rb[2 + k] += fb * B;
  }
  Lb[1] += ppb;
  Rb[1] += ppb;
  const double h0 = 0.5 * Fb[0], h1 = 0.5 * Fb[1];
  const double slb = (Ab + h0) * L[0] + h1 * rel, srb = (Bb + h0) * R[0] + h1 * rer;
  Lb[0] += (Ab + h0) * sl;
  Rb[0] += (Bb + h0) * sr;
  const double relb = h1 * sl, rerb = h1 * sr;
  double vnlb = h1 * L[1] + slb, vnrb = h1 * R[1] + srb;
  Lb[1] += h1 * vnl;
  Rb[1] += h1 * vnr;
  const double rayb = slb - srb;
  // the wave speed of one side: a = sqrt(g p / rho), da = a/2 (dp/p - drho/rho)
  if (right) {
    vnrb += signbit(vnr) ? -rayb : rayb;
    const double h = ad_div(0.5 * rayb * g * iR, ar);
    Rb[1] += h;
    Rb[0] -= h * R[1] * iR;
  } else {
    vnlb += signbit(vnl) ? -rayb : rayb;
    const double h = ad_div(0.5 * rayb * g * iL, al);
    Lb[1] += h;
    Lb[0] -= h * L[1] * iL;
  }
  Lb[1] += relb * ig1;
  Lb[0] += relb * 0.5 * sqL;
  Rb[1] += rerb * ig1;
  Rb[0] += rerb * 0.5 * sqR;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    Lb[2 + k] += relb * L[0] * L[2 + k] + vnlb * n[k];
    Rb[2 + k] += rerb * R[0] * R[2 + k] + vnrb * n[k];
  }
}

// Reverse of flux_hllc_t.
TY_AD void hllc_vjp(double g, const double* L, const double* R, double nx, double ny, double nz,
                    const double* Fb, double* Lb, double* Rb) {
  const double n[3] = {nx, ny, nz};
  const double g1 = g - 1.0, ig1 = ad_rcp(g1), gig1 = g * ig1;
  const double iL = ad_rcp(L[0]), iR = ad_rcp(R[0]);
  const double t1 = ad_sqrt(R[0] * iL), it1 = t1 * L[0] * iR;
  const double kl = ad_rcp(1.0 + t1), kr = t1 * kl;
  double ru[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) ru[k] = kl * L[2 + k] + kr * R[2 + k];
  const double sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4], sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  const double hla = gig1 * L[1] * iL + 0.5 * sqL, hra = gig1 * R[1] * iR + 0.5 * sqR;
  const double h = kl * hla + kr * hra;
  const double H = h - 0.5 * (ru[0] * ru[0] + ru[1] * ru[1] + ru[2] * ru[2]);
  const double vnl = L[2] * nx + L[3] * ny + L[4] * nz, vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  const double al = ad_sqrt(g * L[1] * iL), ar = ad_sqrt(g * R[1] * iR);
  const double vm = ru[0] * nx + ru[1] * ny + ru[2] * nz;
  const double am = ad_sqrt(g1 * H);  // sqrt(g roe_p / roe_rho), roe_p = roe_rho H / gig1
  const double rel = ig1 * L[1] + 0.5 * L[0] * sqL, rer = ig1 * R[1] + 0.5 * R[0] * sqR;
  const bool slm = (vm - am) < (vnl - al), srm = (vm + am) > (vnr + ar);
  const double sl = slm ? vm - am : vnl - al, sr = srm ? vm + am : vnr + ar;
  // adjoints of the intermediate quantities
  double vnlb = 0.0, vnrb = 0.0, relb = 0.0, rerb = 0.0, slb = 0.0, srb = 0.0;
  if (sl >= 0.0 || sr <= 0.0) {  // supersonic: the flux of one side
    const bool lf = sl >= 0.0;
    const double* Q = lf ? L : R;
    double* Qb = lf ? Lb : Rb;
    const double vq = lf ? vnl : vnr, re = lf ? rel : rer;
    const double m0 = vq * Q[0];
    double m0b = Fb[0];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      m0b += Fb[2 + k] * Q[2 + k];
      Qb[2 + k] += Fb[2 + k] * m0;
      Qb[1] += Fb[2 + k] * n[k];
    }
    Qb[1] += Fb[1] * vq;
    Qb[0] += m0b * vq;
    const double vqb = Fb[1] * (re + Q[1]) + m0b * Q[0], reb = Fb[1] * vq;
    if (lf) { vnlb += vqb; relb += reb; } else { vnrb += vqb; rerb += reb; }
  } else {
    const double rqL = L[0] * (sl - vnl), rqR = R[0] * (sr - vnr);
    const double num = rqR * vnr - rqL * vnl - R[1] + L[1], iden = ad_rcp(rqR - rqL);
    const double Sst = num * iden;
    const bool lf = Sst >= 0.0;
    const double* Q = lf ? L : R;
    double* Qb = lf ? Lb : Rb;
    const double s = lf ? sl : sr, vq = lf ? vnl : vnr, rq = lf ? rqL : rqR, re = lf ? rel : rer;
    const double iks = ad_rcp(s - Sst);
    const double rst = rq * iks;
    const double pst = Q[1] - rq * (vq - Sst);
    const double dp = pst - Q[1];
    double M[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) M[k] = rq * Q[2 + k] + dp * n[k];
    const double E = re * (s - vq) - Q[1] * vq + pst * Sst;
    const double rest = iks * E;
    double Sstb = Fb[0] * rst + Fb[1] * (rest + pst);
    const double rstb = Fb[0] * Sst, restb = Fb[1] * Sst;
    double pstb = Fb[1] * Sst;
    double iksb = restb * E, rqb = 0.0, dpb = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      Sstb += Fb[2 + k] * iks * M[k];
      pstb += Fb[2 + k] * n[k];
      const double Mb = Fb[2 + k] * Sst * iks;
      iksb += Fb[2 + k] * Sst * M[k];
      rqb += Mb * Q[2 + k];
      Qb[2 + k] += Mb * rq;
      dpb += Mb * n[k];
    }
    const double Eb = restb * iks;
    double sb = Eb * re, vqb = -Eb * (re + Q[1]), pQb = -Eb * vq;
    const double reb = Eb * (s - vq);
    pstb += Eb * Sst + dpb;
    Sstb += Eb * pst;
    pQb += pstb - dpb;
    rqb += -pstb * (vq - Sst) + rstb * iks;
    vqb -= pstb * rq;
    Sstb += pstb * rq;
    iksb += rstb * rq;
    sb -= iksb * iks * iks;
    Sstb += iksb * iks * iks;
    Qb[1] += pQb;
    double rqLb = 0.0, rqRb = 0.0;
    if (lf) { vnlb += vqb; relb += reb; slb += sb; rqLb = rqb; }
    else { vnrb += vqb; rerb += reb; srb += sb; rqRb = rqb; }
    const double numb = Sstb * iden, denb = -Sstb * Sst * iden;
    rqRb += numb * vnr + denb;
    rqLb += -numb * vnl - denb;
    vnrb += numb * rqR;
    vnlb -= numb * rqL;
    Rb[1] -= numb;
    Lb[1] += numb;
    Lb[0] += rqLb * (sl - vnl);
    slb += rqLb * L[0];
    vnlb -= rqLb * L[0];
    Rb[0] += rqRb * (sr - vnr);
    srb += rqRb * R[0];
    vnrb -= rqRb * R[0];
  }
  // wave speeds
  double vmb = 0.0, amb = 0.0, alb = 0.0, arb = 0.0;
  if (slm) { vmb += slb; amb -= slb; } else { vnlb += slb; alb -= slb; }
  if (srm) { vmb += srb; amb += srb; } else { vnrb += srb; arb += srb; }
  // am = sqrt(g1 H): dam = g1 / (2 am) dH (the Roe density cancels)
  const double Hb = ad_div(amb * 0.5 * g1, am);
  double klb = Hb * hla, krb = Hb * hra;
  const double hlab = Hb * kl, hrab = Hb * kr;
  const double sqLb = 0.5 * hlab + relb * 0.5 * L[0], sqRb = 0.5 * hrab + rerb * 0.5 * R[0];
  const double alh = ad_div(alb * 0.5 * g * iL, al), arh = ad_div(arb * 0.5 * g * iR, ar);
  Lb[1] += hlab * gig1 * iL + relb * ig1 + alh;
  Lb[0] += relb * 0.5 * sqL - (hlab * gig1 * iL + alh) * L[1] * iL;
  Rb[1] += hrab * gig1 * iR + rerb * ig1 + arh;
  Rb[0] += rerb * 0.5 * sqR - (hrab * gig1 * iR + arh) * R[1] * iR;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double rub = vmb * n[k] - Hb * ru[k];
    klb += rub * L[2 + k];
    krb += rub * R[2 + k];
    Lb[2 + k] += rub * kl + 2.0 * sqLb * L[2 + k] + vnlb * n[k];
    Rb[2 + k] += rub * kr + 2.0 * sqRb * R[2 + k] + vnrb * n[k];
  }
  double t1b = krb * kl;
  klb += krb * t1;
  t1b -= klb * kl * kl;
  const double rb = t1b * 0.5 * it1;  // t1 = sqrt(R0 / L0)
  Rb[0] += rb * iL;
  Lb[0] -= rb * R[0] * iL * iL;
}

}  // namespace adflux
}  // namespace tyk
