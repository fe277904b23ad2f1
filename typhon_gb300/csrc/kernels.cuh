// Kernels of the explicit residual-and-update path, compiled once per arithmetic mode.
//
// Included by kernels_exact.cu (TY_KNS = kexact, TY_FAST = 0, compiled with -fmad=false:
// every FP64 operation separately rounded, in Typhon's order) and kernels_fast.cu
// (TY_KNS = kfast, TY_FAST = 1, fused multiply-add and precomputed weights).
//
// Typhon routines restated (file:line of the Fortran reference):
//   k_prim          SOURCE/EQNS/calc_varprim_ns.f90:43-54
//   k_ghost_prim    SOURCE/MGRID/calcboco_connect_per_match.f90:56-78 (periodic copy),
//                   SOURCE/MGRID/calcboco_ust_sym.f90 (symmetry mirror)
//   k_grad          SOURCE/MGRID/calc_gradient.f90:67-196 + SOURCE/MATH/MATRIX.f90:79-111
//   k_ghost_grad    SOURCE/MGRID/calcboco_gen.f90:78-84 (connections only)
//   recon           SOURCE/EQNS/hres_ns_musclfast.f90, hres_ns_muscl.f90, hres_ns_muscluns.f90,
//                   tvdgrad{fst,str,uns}_{scal,vect}.f90, SOURCE/MGRID/LIMITER.f90
//   k_barth         SOURCE/MGRID/postlimit_barth.f90:42-223
//   flux_*          SOURCE/EQNS/calc_flux_hllc.f90:61-171, calc_roe_states.f90:35-53,
//                   calc_flux_rusanov.f90:57-83; Roe: new (Roe 1981 + Harten fix)
//   k_gather        SOURCE/MAIN/flux_to_res.f90:47-144 (colour-ordered sums, as a gather)
//   k_rk_update     SOURCE/MAIN/treelevel_rungekutta.f90:60-113, SOURCE/ZONE/update_field.f90:38
//   k_timestep      SOURCE/EQNS/calc_ns_timestep.f90:52-103
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/typhon_gpu.h"
#include "devmesh.hpp"
#include "fastmath.cuh"

#ifndef TY_KNS
#error "define TY_KNS and TY_FAST before including kernels.cuh"
#endif

namespace tyk {
namespace TY_KNS {

constexpr bool kFast = TY_FAST;
constexpr int kBlock = 256;

__device__ __forceinline__ double d3(const double* a, int ld, int i, int k) { return a[k * (size_t)ld + i]; }

// Rotational periodicity (calcboco_connect_per_match.f90:56-78, transvec_per): the velocity
// (q[2..4]) of a state taken from the partner of periodic face f, rotated into f's frame.
__device__ __forceinline__ void rot_to_face(const DevMesh& m, int f, double* q) {
  if (!m.frot) return;
  const size_t lf = m.ldf;
  double R[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = m.frot[k * lf + f];
  const double x = q[2], y = q[3], z = q[4];
  q[2] = R[0] * x + R[1] * y + R[2] * z;
  q[3] = R[3] * x + R[4] * y + R[5] * z;
  q[4] = R[6] * x + R[7] * y + R[8] * z;
}

// ---------------------------------------------------------------------------
// Limiters (LIMITER.f90).  Scalars (rho, p) pass through the array forms, vector
// components through the scalar forms, as tvdgrad*_scal / tvdgrad*_vect call them.
__device__ __forceinline__ double sgn1(double x) { return signbit(x) ? -1.0 : 1.0; }

__device__ double lim_scalar_form(int lim, double x1, double x2) {
  switch (lim) {
    case TY_LIM_MINMOD: {
      double s = 0.5 * (sgn1(x1) + sgn1(x2));
      return s * fmin(fabs(x1), fabs(x2));
    }
    case TY_LIM_ALBADA: {
      double s = x1 * x2;
      if (s <= 0.0) return 0.0;
      return s * (x1 + x2) / (x1 * x1 + x2 * x2);
    }
    case TY_LIM_VLEER: {
      double s = x1 * x2;
      if (s <= 0.0) return 0.0;
      return 2.0 * s / (x1 + x2);
    }
    case TY_LIM_SUPERBEE: {
      double r = 0.0;
      if (x1 > 0.0 && x2 > 0.0) r = fmax(fmin(2.0 * x1, x2), fmin(2.0 * x2, x1));
      if (x1 < 0.0 && x2 < 0.0) r = fmin(fmax(2.0 * x1, x2), fmax(2.0 * x2, x1));
      return r;
    }
    case TY_LIM_KIM3: {
      double r = 0.0;
      if (x1 > 0.0 && x2 > 0.0) { r = (2.0 * x1 + x2) / 3.0; r = fmin(fmin(2.0 * x1, 2.0 * x2), r); }
      if (x1 < 0.0 && x2 < 0.0) { r = (2.0 * x1 + x2) / 3.0; r = fmax(fmax(2.0 * x1, 2.0 * x2), r); }
      return r;
    }
    case TY_LIM_LIM03: {
      double eta = (x1 * x1 + x2 * x2) / 0.01 / 0.01;
      double r = 0.0;
      if (eta < 1.0) r = (2.0 * x2 + x1) / 3.0;
      else if (x1 > 0.0 && x2 > 0.0) { r = (2.0 * x2 + x1) / 3.0; r = fmin(fmin(1.6 * x2, 2.0 * x1), r); }
      else if (x1 < 0.0 && x2 < 0.0) { r = (2.0 * x2 + x1) / 3.0; r = fmax(fmax(1.6 * x2, 2.0 * x1), r); }
      else if (x1 < 0.0 && x2 > 0.0) { r = (2.0 * x2 + x1) / 3.0; r = fmax(0.0, fmin(-0.5 * x1, r)); }
      else if (x1 > 0.0 && x2 < 0.0) { r = (2.0 * x2 + x1) / 3.0; r = fmin(0.0, fmax(-0.5 * x1, r)); }
      return r;
    }
  }
  return 0.0;
}
__device__ double lim_array_form(int lim, double x1, double x2) {
  switch (lim) {
    case TY_LIM_MINMOD:
      if (x1 > 0.0 && x2 > 0.0) return fmin(x1, x2);
      if (x1 < 0.0 && x2 < 0.0) return fmax(x1, x2);
      return 0.0;
    case TY_LIM_ALBADA:
      if ((x1 > 0.0 && x2 > 0.0) || (x1 < 0.0 && x2 < 0.0)) return x1 * x2 * (x1 + x2) / (x1 * x1 + x2 * x2);
      return 0.0;
    case TY_LIM_VLEER:
      if ((x1 > 0.0 && x2 > 0.0) || (x1 < 0.0 && x2 < 0.0)) return 2.0 * x1 * x2 / (x1 + x2);
      return 0.0;
    default:
      return lim_scalar_form(lim, x1, x2);
  }
}
// slope limiter of the MUSCL variants: lim(2g - LR, LR) for FAST/str, lim(g, LR) for UNS;
// KIM3 takes its arguments swapped
__device__ __forceinline__ double apply_lim(int lim, bool uns, bool arrayform, double g, double LR) {
  double a = uns ? g : 2.0 * g - LR, b = LR;
  if (lim == TY_LIM_KIM3) { double t = a; a = b; b = t; }
  return arrayform ? lim_array_form(lim, a, b) : lim_scalar_form(lim, a, b);
}

// ---------------------------------------------------------------------------
// cons -> prim (calc_varprim_ns.f90:43-54)
__device__ __forceinline__ void cons_to_prim(double gamma, const double c[5], double q[5]) {
  const double g1 = gamma - 1.0;
  double rho = c[0];
  double vx, vy, vz;
  if constexpr (kFast) {
    const double ir = rcp_nr(rho);
    vx = c[2] * ir; vy = c[3] * ir; vz = c[4] * ir;
  } else {
    vx = c[2] / rho; vy = c[3] / rho; vz = c[4] / rho;
  }
  double ec = 0.5 * rho * (vx * vx + vy * vy + vz * vz);
  q[0] = rho;
  q[1] = g1 * (c[1] - ec);
  q[2] = vx; q[3] = vy; q[4] = vz;
}

__global__ void k_prim(DevMesh m, const double* __restrict__ cons, double* __restrict__ prim, double gamma) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  double u[5], q[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) u[v] = cons[v * (size_t)m.ldc + c];
  cons_to_prim(gamma, u, q);
#pragma unroll
  for (int v = 0; v < 5; ++v) prim[v * (size_t)m.ldc + c] = q[v];
}

// calc_viscosity (SOURCE/EQNS/EQNS.f90:225-265): nu rho, or Sutherland with AIR's constants
__device__ __forceinline__ double viscosity(const SpatOpts& o, double rho, double T) {
  if (o.visc_law == TY_VISC_KINEMATIC) return o.visc_kin * rho;
  const double mu0 = 0.0000168, T0 = 273.00, S = 110.50;
  return mu0 * pow(T / T0, 1.5) * (T0 + S) / (T + S);
}

// far-field ghost state (new), kind fixed by the free-stream normal velocity (see ty_bc)
__device__ __forceinline__ void farfield_state(const SpatOpts& o, double nx, double ny, double nz, const double* q,
                                               double* out) {
  const double* qi = o.farfield;
  const double vn = qi[2] * nx + qi[3] * ny + qi[4] * nz;
  const double c = sqrt(o.gamma * qi[1] / qi[0]);
  if (vn <= -c) {
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v] = qi[v];
  } else if (vn < -1e-8 * c) {
    out[0] = qi[0]; out[1] = q[1]; out[2] = qi[2]; out[3] = qi[3]; out[4] = qi[4];
  } else if (vn < c) {
    out[0] = q[0]; out[1] = qi[1]; out[2] = q[2]; out[3] = q[3]; out[4] = q[4];
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v] = q[v];
  }
}

// inlet / outlet states from the inside state qi (setboco_ns_inlet_sub.f90:64-96,
// setboco_ns_outlet_sub.f90:31-60, setboco_ns_inlet_sup.f90:75-101, setboco_ns_outlet_sup.f90)
// with the isentropic relations of EQNS.f90:139-219 (pi_ti_mach_dir2nspri,
// pi_ti_ps_dir2nspri, nspri2pi_ti_mach_dir), in their operation order
__device__ void inout_state(const DevMesh& m, const SpatOpts& o, int f, int kind, const double* qi, double* qo) {
  if (kind == TY_BC_OUTLET_SUP) {
#pragma unroll
    for (int v = 0; v < 5; ++v) qo[v] = qi[v];
    return;
  }
  const double g = o.gamma, r = o.rgas, g1 = g - 1.0;
  const size_t lf = m.ldf;
  const double* D = m.fbcd + f;
  if (kind == TY_BC_INLET_SUP) {
    const double dx = D[3 * lf], dy = D[4 * lf], dz = D[5 * lf];
    const double dn = sqrt(dx * dx + dy * dy + dz * dz);
    const double mach = D[2 * lf];
    const double fm = 1.0 / (1.0 + .5 * g1 * (mach * mach));
    const double ts = D[lf] * fm;
    const double a = sqrt(g * r * ts);
    qo[1] = D[0] * pow(fm, g / g1);
    qo[0] = qo[1] / (r * ts);
    const double va = mach * a;
    qo[2] = va * (dx / dn); qo[3] = va * (dy / dn); qo[4] = va * (dz / dn);
    return;
  }
  double pi, ti, ps, ux, uy, uz;
  if (kind == TY_BC_INLET_SUB) {
    pi = D[0]; ti = D[lf]; ps = qi[1];
    const double dx = D[2 * lf], dy = D[3 * lf], dz = D[4 * lf];
    const double dn = sqrt(dx * dx + dy * dy + dz * dz);
    ux = dx / dn; uy = dy / dn; uz = dz / dn;
  } else {  // TY_BC_OUTLET_SUB: totals and direction of the inside state
    double fmv = qi[2] * qi[2] + qi[3] * qi[3] + qi[4] * qi[4];
    const double n = sqrt(fmv);
    ux = qi[2] / n; uy = qi[3] / n; uz = qi[4] / n;
    fmv = fmv / (g * qi[1]) * qi[0];
    fmv = 1.0 + 0.5 * g1 * fmv;
    pi = qi[1] * pow(fmv, g / g1);
    ti = qi[1] / r / qi[0] * fmv;
    ps = D[0];
  }
  double fm = pow(pi / ps, g1 / g);
  if (fm < 1.0) fm = 1.0;  // Typhon: "Bad ratio Pi/P : truncated to 1."
  qo[1] = ps;
  qo[0] = ps / (r * ti) * fm;
  const double va = sqrt((fm - 1.0) * 2.0 / g1) * sqrt(g * ps / qo[0]);
  qo[2] = va * ux; qo[3] = va * uy; qo[4] = va * uz;
}

// ghost states: periodic copy, symmetry mirror (velocity reflected across the face),
// adiabatic moving wall (setboco_ns_flux.f90, cell-state mode: pressure copied, temperature
// of the cell minus lflux d / conduct with lflux = 0, velocity reflected about the wall's)
__global__ void k_ghost_prim(DevMesh m, double* __restrict__ prim, SpatOpts o) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m.ng) return;
  const int g = m.nci + k, src = m.gsrc[k], f = m.gface[k];
  const size_t ld = m.ldc;
  const int kind = m.fbc[f];
  double vx = prim[2 * ld + src], vy = prim[3 * ld + src], vz = prim[4 * ld + src];
  if (kind == TY_BC_FARFIELD || kind >= TY_BC_INLET_SUB) {
    double q[5], out[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) q[v] = prim[v * ld + src];
    if (kind == TY_BC_FARFIELD)
      farfield_state(o, d3(m.fn, m.ldf, f, 0), d3(m.fn, m.ldf, f, 1), d3(m.fn, m.ldf, f, 2), q, out);
    else
      inout_state(m, o, f, kind, q, out);
#pragma unroll
    for (int v = 0; v < 5; ++v) prim[v * ld + g] = out[v];
    return;
  }
  if (kind == TY_BC_WALL || kind == TY_BC_NOSLIP) {
    const double r = o.rgas, lflux = 0.0;
    const double rho = prim[src], p = prim[ld + src];
    const double mu = viscosity(o, rho, p / (r * rho));
    const double cp = o.gamma / (o.gamma - 1.0) * r;
    const double conduct = mu * cp / o.prandtl;
    const double temp = p / (rho * r) - lflux * m.gdist[k] / conduct;
    prim[ld + g] = p;
    prim[g] = p / (r * temp);
    prim[2 * ld + g] = (2.0 * d3(m.fwall, m.ldf, f, 0)) - vx;
    prim[3 * ld + g] = (2.0 * d3(m.fwall, m.ldf, f, 1)) - vy;
    prim[4 * ld + g] = (2.0 * d3(m.fwall, m.ldf, f, 2)) - vz;
    return;
  }
  prim[g] = prim[src];
  prim[ld + g] = prim[ld + src];
  if (kind == TY_BC_PERIODIC && m.frot) {
    double q[5] = {0.0, 0.0, vx, vy, vz};
    rot_to_face(m, f, q);
    vx = q[2]; vy = q[3]; vz = q[4];
  }
  if (kind == TY_BC_SYMMETRY) {
    double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
    double wx = vx - 0.0, wy = vy - 0.0, wz = vz - 0.0;
    double dn = 2.0 * (wx * nx + wy * ny + wz * nz);
    vx = vx - dn * nx; vy = vy - dn * ny; vz = vz - dn * nz;
  }
  prim[2 * ld + g] = vx;
  prim[3 * ld + g] = vy;
  prim[4 * ld + g] = vz;
}

// ---------------------------------------------------------------------------
// least-squares gradient: b_c = sum_f (q(fc2) - q(fc1)) d_f over the cell's faces in colour
// order, then the Cholesky solve (exact) or, in fast mode, the precomputed A^-1 d weights.
__global__ void __launch_bounds__(kBlock) k_grad(DevMesh m, DevState s) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t ld = m.ldc;
  double b[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) b[k] = 0.0;
  const double* __restrict__ prim = s.prim;
  for (int sl = 0; sl < m.nslot; ++sl) {
    int e = m.cf[sl * (size_t)m.nci + c];
    if (e < 0) break;
    int f = e >> 1;
    int i1 = m.fc1[f], i2 = m.fc2[f];
    if constexpr (kFast) {
      const int side = e & 1;
      const double wx = d3(m.lsqw, m.ldf, f, 3 * side), wy = d3(m.lsqw, m.ldf, f, 3 * side + 1),
                   wz = d3(m.lsqw, m.ldf, f, 3 * side + 2);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double dsca = prim[v * ld + i2] - prim[v * ld + i1];
        b[3 * v] = fma(dsca, wx, b[3 * v]);
        b[3 * v + 1] = fma(dsca, wy, b[3 * v + 1]);
        b[3 * v + 2] = fma(dsca, wz, b[3 * v + 2]);
      }
    } else {
      const double dx = d3(m.dcg, m.ldf, f, 0), dy = d3(m.dcg, m.ldf, f, 1), dz = d3(m.dcg, m.ldf, f, 2);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double dsca = prim[v * ld + i2] - prim[v * ld + i1];
        b[3 * v] = b[3 * v] + dsca * dx;
        b[3 * v + 1] = b[3 * v + 1] + dsca * dy;
        b[3 * v + 2] = b[3 * v + 2] + dsca * dz;
      }
    }
  }
  if constexpr (!kFast) {
    const double L11 = m.lsq[c], L21 = m.lsq[m.nci + c], L31 = m.lsq[2 * (size_t)m.nci + c];
    const double L22 = m.lsq[3 * (size_t)m.nci + c], L32 = m.lsq[4 * (size_t)m.nci + c];
    const double L33 = m.lsq[5 * (size_t)m.nci + c];
    // cholesky_solve (MATRIX.f90:79-111), column per variable
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double x1 = b[3 * v], x2 = b[3 * v + 1], x3 = b[3 * v + 2];
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
      b[3 * v] = x1; b[3 * v + 1] = x2; b[3 * v + 2] = x3;
    }
  }
#pragma unroll
  for (int k = 0; k < 15; ++k) s.grad[k * ld + c] = b[k];
}

__global__ void k_ghost_grad(DevMesh m, double* __restrict__ grad) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m.ng) return;
  const int f = m.gface[k];
  if (m.fbc[f] != TY_BC_PERIODIC) return;
  const int g = m.nci + k, src = m.gsrc[k];
  const size_t ld = m.ldc;
  if (!m.frot) {
#pragma unroll
    for (int v = 0; v < 15; ++v) grad[v * ld + g] = grad[v * ld + src];
    return;
  }
  // rotational periodicity: the scalar gradients are vectors, R g (transvec_per); the velocity
  // gradient G(i,j) = du_i/dx_j becomes G R^T (transten_per -> t3d_rot, TENSOR3.f90:328-340)
  const size_t lf = m.ldf;
  double R[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) R[q] = m.frot[q * lf + f];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const double x = grad[(3 * q) * ld + src], y = grad[(3 * q + 1) * ld + src], z = grad[(3 * q + 2) * ld + src];
    grad[(3 * q) * ld + g] = R[0] * x + R[1] * y + R[2] * z;
    grad[(3 * q + 1) * ld + g] = R[3] * x + R[4] * y + R[5] * z;
    grad[(3 * q + 2) * ld + g] = R[6] * x + R[7] * y + R[8] * z;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double G0 = grad[(6 + 3 * i) * ld + src], G1 = grad[(7 + 3 * i) * ld + src], G2 = grad[(8 + 3 * i) * ld + src];
#pragma unroll
    for (int j = 0; j < 3; ++j) grad[(6 + 3 * i + j) * ld + g] = G0 * R[3 * j] + G1 * R[3 * j + 1] + G2 * R[3 * j + 2];
  }
}

// ---------------------------------------------------------------------------
// High-order face state on one side of face f (side 0: cell fc1 "L", side 1: cell fc2 "R").
__device__ void recon(const DevMesh& m, const DevState& s, const SpatOpts& o, int f, int side, double q[5]) {
  const size_t ld = m.ldc;
  const int icl = m.fc1[f], icr = m.fc2[f];
  const int c = side ? icr : icl;
  const double* __restrict__ prim = s.prim;
#pragma unroll
  for (int v = 0; v < 5; ++v) q[v] = prim[v * ld + c];
  if (o.highres == TY_HRES_NONE) return;
  const double* __restrict__ gr = s.grad;
  const double ux = d3(m.uLR, m.ldf, f, 0), uy = d3(m.uLR, m.ldf, f, 1), uz = d3(m.uLR, m.ldf, f, 2);
  const double dLR = m.dLR[f];
  if (o.highres == TY_HRES_MUSCLFAST) {
    const double k = side ? m.kRF[f] : m.kLF[f];
    // scalars (tvdgradfst_scal.f90:35-57)
#pragma unroll
    for (int sv = 0; sv < 2; ++sv) {
      double LR = (prim[sv * ld + icr] - prim[sv * ld + icl]) / dLR;
      double sg;
      if (o.limiter == TY_LIM_NONE) {
        sg = LR;
      } else {
        double g = gr[(3 * sv) * ld + c] * ux + gr[(3 * sv + 1) * ld + c] * uy + gr[(3 * sv + 2) * ld + c] * uz;
        sg = apply_lim(o.limiter, false, true, g, LR);
      }
      q[sv] = q[sv] + sg * k;
    }
    // velocity (tvdgradfst_vect.f90:36-58)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double LR = (prim[(2 + i) * ld + icr] - prim[(2 + i) * ld + icl]) / dLR;
      double sg;
      if (o.limiter == TY_LIM_NONE) {
        sg = LR;
      } else {
        double g = gr[(6 + 3 * i) * ld + c] * ux + gr[(7 + 3 * i) * ld + c] * uy + gr[(8 + 3 * i) * ld + c] * uz;
        sg = apply_lim(o.limiter, false, false, g, LR);
      }
      q[2 + i] = q[2 + i] + k * sg;
    }
    return;
  }
  // MUSCL / MUSCL-UNS (tvdgradstr_*.f90, tvdgraduns_*.f90)
  const bool uns = o.highres == TY_HRES_MUSCLUNS;
  const double* CF = side ? m.RF : m.LF;
  const double cx = d3(CF, m.ldf, f, 0), cy = d3(CF, m.ldf, f, 1), cz = d3(CF, m.ldf, f, 2);
#pragma unroll
  for (int sv = 0; sv < 2; ++sv) {
    double LR = (prim[sv * ld + icr] - prim[sv * ld + icl]) / dLR;
    double gx = gr[(3 * sv) * ld + c], gy = gr[(3 * sv + 1) * ld + c], gz = gr[(3 * sv + 2) * ld + c];
    double g = gx * ux + gy * uy + gz * uz;
    double sg = o.limiter == TY_LIM_NONE ? LR - g : apply_lim(o.limiter, uns, true, g, LR) - g;
    gx = gx + sg * ux; gy = gy + sg * uy; gz = gz + sg * uz;
    q[sv] = q[sv] + (gx * cx + gy * cy + gz * cz);
  }
  double T[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) T[k] = gr[(6 + k) * ld + c];
  double sgv[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double LR = (prim[(2 + i) * ld + icr] - prim[(2 + i) * ld + icl]) / dLR;
    double g = T[3 * i] * ux + T[3 * i + 1] * uy + T[3 * i + 2] * uz;
    sgv[i] = o.limiter == TY_LIM_NONE ? LR - g : apply_lim(o.limiter, uns, false, g, LR) - g;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double t0 = T[3 * i] + sgv[i] * ux, t1 = T[3 * i + 1] + sgv[i] * uy, t2 = T[3 * i + 2] + sgv[i] * uz;
    q[2 + i] = q[2 + i] + (t0 * cx + t1 * cy + t2 * cz);
  }
}

// moving adiabatic wall, face-state mode (setboco_ns_flux.f90): the right state takes the left
// state's pressure as its density, its pressure, and the velocity reflected about the wall's
__device__ __forceinline__ void wall_state(const DevMesh& m, int f, const double* QL, double* QR) {
  QR[0] = m.fbc[f] == TY_BC_NOSLIP ? QL[0] : QL[1];  // TY_BC_NOSLIP: the inside density (new)
  QR[1] = QL[1];
  QR[2] = (2.0 * d3(m.fwall, m.ldf, f, 0)) - QL[2];
  QR[3] = (2.0 * d3(m.fwall, m.ldf, f, 1)) - QL[3];
  QR[4] = (2.0 * d3(m.fwall, m.ldf, f, 2)) - QL[4];
}

// velocity mirrored across the face plane (calcboco_ust_sym.f90, face-state mode)
__device__ __forceinline__ void mirror(const DevMesh& m, int f, double q[5]) {
  double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  double wx = q[2] - 0.0, wy = q[3] - 0.0, wz = q[4] - 0.0;
  double dn = 2.0 * (wx * nx + wy * ny + wz * nz);
  q[2] = q[2] - dn * nx; q[3] = q[3] - dn * ny; q[4] = q[4] - dn * nz;
}

// ---------------------------------------------------------------------------
// Riemann fluxes per unit area, F = (mass, energy, momentum x, y, z)

// Outer wave speeds of the HLL family (calc_flux_hllc.f90:64-124, calc_flux_hlle.f90:64-120):
// beta = 1 (HLLC, HLLE, K) or sqrt((g-1)/(2g)) (B, KB variants); the kinetic variants take the
// EFM estimates c (m kinw + kind), m = vn/c -+ f1 beta, c = a/f1, kinw = (1 -+ erf m)/2,
// kind = -+ f2 exp(-m^2).  Standard HLLE speeds are clamped to 0, the kinetic ones are not.
__device__ __forceinline__ void hll_speeds(const SpatOpts& o, double vnl, double vnr, double al, double ar, double vm,
                                           double am, double& sl, double& sr) {
  const double beta = o.hll_beta;
  if (o.hll_kin) {
    const double f1 = o.hll_f1, f2 = o.hll_f2;
    const double cl = al / f1, cr = ar / f1;
    const double modml = vnl / cl - f1 * beta, modmr = vnr / cr + f1 * beta;
    const double kinwl = 0.5 * (1.0 - erf(modml)), kinwr = 0.5 * (1.0 + erf(modmr));
    const double kindl = -f2 * exp(-modml * modml), kindr = +f2 * exp(-modmr * modmr);
    sl = fmin(cl * (modml * kinwl + kindl), vm - am);
    sr = fmax(cr * (modmr * kinwr + kindr), vm + am);
  } else if (o.hll_family == 2) {
    sl = fmin(fmin(0.0, vnl - beta * al), vm - am);
    sr = fmax(fmax(0.0, vnr + beta * ar), vm + am);
  } else {
    sl = fmin(vnl - beta * al, vm - am);
    sr = fmax(vnr + beta * ar, vm + am);
  }
}

// calc_flux_hlle.f90:83-150 (beta = 1), the Roe average of calc_roe_states.f90:37-53
__device__ void flux_hlle(const SpatOpts& o, const double* L, const double* R, double nx, double ny, double nz,
                          double* F) {
  const double g = o.gamma;
  const double ig1 = 1.0 / (g - 1.0);
  const double gig1 = g / (g - 1.0);
  double t1 = sqrt(R[0] / L[0]);
  double roe_rho = L[0] * t1;
  double kl0 = 1.0 / (1.0 + t1);
  double kr0 = t1 * kl0;
  double rux = kl0 * L[2] + kr0 * R[2], ruy = kl0 * L[3] + kr0 * R[3], ruz = kl0 * L[4] + kr0 * R[4];
  double sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4];
  double sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  double h1 = gig1 * L[1] / L[0] + 0.5 * sqL;
  double h2 = gig1 * R[1] / R[0] + 0.5 * sqR;
  h1 = kl0 * h1 + kr0 * h2;
  double roe_p = (h1 - 0.5 * (rux * rux + ruy * ruy + ruz * ruz)) * roe_rho / gig1;
  double vnl = L[2] * nx + L[3] * ny + L[4] * nz;
  double vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  double al = sqrt(g * L[1] / L[0]);
  double ar = sqrt(g * R[1] / R[0]);
  double vm = rux * nx + ruy * ny + ruz * nz;
  double am = sqrt(g * roe_p / roe_rho);
  double rel = ig1 * L[1] + .5 * L[0] * sqL;
  double rer = ig1 * R[1] + .5 * R[0] * sqR;
  double sl, sr;
  hll_speeds(o, vnl, vnr, al, ar, vm, am, sl, sr);
  double iks = 1.0 / (sr - sl);
  double kl = sr * iks, kr = -sl * iks, ku = sl * sr * iks;
  double wl = kl * vnl - ku, wr = kr * vnr + ku;
  F[0] = wl * L[0] + wr * R[0];
  F[1] = wl * rel + wr * rer + (kl * vnl * L[1] + kr * vnr * R[1]);
  double ml = wl * L[0], mr = wr * R[0], pp = kl * L[1] + kr * R[1];
  F[2] = ml * L[2] + mr * R[2] + pp * nx;
  F[3] = ml * L[3] + mr * R[3] + pp * ny;
  F[4] = ml * L[4] + mr * R[4] + pp * nz;
}
// calc_flux_ausmm.f90:62-118: AUSM-M, van Leer's Mach and pressure splittings (no Jacobian)
__device__ void flux_ausmm(double g, const double* L, const double* R, double nx, double ny, double nz, double* F) {
  const double gig1 = g / (g - 1.0);
  const double al = sqrt(g * L[1] / L[0]);
  const double ar = sqrt(g * R[1] / R[0]);
  const double mnl = (L[2] * nx + L[3] * ny + L[4] * nz) / al;
  const double mnr = (R[2] * nx + R[3] * ny + R[4] * nz) / ar;
  double mp, pp, mm, pm;
  if (mnl >= 1.0) { mp = mnl; pp = 1.0; }
  else if (mnl <= -1.0) { mp = 0.0; pp = 0.0; }
  else { mp = .25 * ((mnl + 1.0) * (mnl + 1.0)); pp = mp * (2.0 - mnl); }
  if (mnr <= -1.0) { mm = mnr; pm = 1.0; }
  else if (mnr >= 1.0) { mm = 0.0; pm = 0.0; }
  else { mm = -(.25 * ((mnr - 1.0) * (mnr - 1.0))); pm = -mm * (2.0 + mnr); }
  const double ms = mp + mm;
  const double wl = al * fmax(0.0, ms), wr = ar * fmin(0.0, ms);
  const double rhl = gig1 * L[1] + .5 * L[0] * (L[2] * L[2] + L[3] * L[3] + L[4] * L[4]);
  const double rhr = gig1 * R[1] + .5 * R[0] * (R[2] * R[2] + R[3] * R[3] + R[4] * R[4]);
  F[0] = wl * L[0] + wr * R[0];
  F[1] = wl * rhl + wr * rhr;
  const double ml = wl * L[0], mr = wr * R[0], pf = pp * L[1] + pm * R[1];
  F[2] = ml * L[2] + mr * R[2] + pf * nx;
  F[3] = ml * L[3] + mr * R[3] + pf * ny;
  F[4] = ml * L[4] + mr * R[4] + pf * nz;
}
__device__ void flux_hllc(const SpatOpts& o, const double* L, const double* R, double nx, double ny, double nz,
                          double* F) {
  const double g = o.gamma;
  const double ig1 = 1.0 / (g - 1.0);
  const double gig1 = g / (g - 1.0);
  // calc_roe_states.f90:37-53
  double t1 = sqrt(R[0] / L[0]);
  double roe_rho = L[0] * t1;
  double kl = 1.0 / (1.0 + t1);
  double kr = t1 * kl;
  double rux = kl * L[2] + kr * R[2], ruy = kl * L[3] + kr * R[3], ruz = kl * L[4] + kr * R[4];
  double sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4];
  double sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  double h1 = gig1 * L[1] / L[0] + 0.5 * sqL;
  double h2 = gig1 * R[1] / R[0] + 0.5 * sqR;
  h1 = kl * h1 + kr * h2;
  double roe_p = (h1 - 0.5 * (rux * rux + ruy * ruy + ruz * ruz)) * roe_rho / gig1;
  // calc_flux_hllc.f90:86-171 (beta = 1)
  double vnl = L[2] * nx + L[3] * ny + L[4] * nz;
  double vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  double al = sqrt(g * L[1] / L[0]);
  double ar = sqrt(g * R[1] / R[0]);
  double vm = rux * nx + ruy * ny + ruz * nz;
  double am = sqrt(g * roe_p / roe_rho);
  double rel = ig1 * L[1] + 0.5 * L[0] * sqL;
  double rer = ig1 * R[1] + 0.5 * R[0] * sqR;
  double sl, sr;
  hll_speeds(o, vnl, vnr, al, ar, vm, am, sl, sr);
  if (sl >= 0.0) {
    F[0] = vnl * L[0];
    F[1] = vnl * (rel + L[1]);
    double m0 = vnl * L[0];
    F[2] = m0 * L[2] + L[1] * nx; F[3] = m0 * L[3] + L[1] * ny; F[4] = m0 * L[4] + L[1] * nz;
  } else if (sr <= 0.0) {
    F[0] = vnr * R[0];
    F[1] = vnr * (rer + R[1]);
    double m0 = vnr * R[0];
    F[2] = m0 * R[2] + R[1] * nx; F[3] = m0 * R[3] + R[1] * ny; F[4] = m0 * R[4] + R[1] * nz;
  } else {
    double rqL = L[0] * (sl - vnl);
    double rqR = R[0] * (sr - vnr);
    double Sst = (rqR * vnr - rqL * vnl - R[1] + L[1]) / (rqR - rqL);
    double iks, rst, pst, rest, rvx, rvy, rvz;
    if (Sst >= 0.0) {
      iks = 1.0 / (sl - Sst);
      rst = rqL * iks;
      pst = L[1] - rqL * (vnl - Sst);
      double dp = pst - L[1];
      rvx = iks * ((rqL * L[2]) + dp * nx); rvy = iks * ((rqL * L[3]) + dp * ny); rvz = iks * ((rqL * L[4]) + dp * nz);
      rest = iks * (rel * (sl - vnl) - L[1] * vnl + pst * Sst);
    } else {
      iks = 1.0 / (sr - Sst);
      rst = rqR * iks;
      pst = R[1] - rqR * (vnr - Sst);
      double dp = pst - R[1];
      rvx = iks * ((rqR * R[2]) + dp * nx); rvy = iks * ((rqR * R[3]) + dp * ny); rvz = iks * ((rqR * R[4]) + dp * nz);
      rest = iks * (rer * (sr - vnr) - R[1] * vnr + pst * Sst);
    }
    F[0] = Sst * rst;
    F[1] = Sst * (rest + pst);
    F[2] = (Sst * rvx) + (pst * nx); F[3] = (Sst * rvy) + (pst * ny); F[4] = (Sst * rvz) + (pst * nz);
  }
}

__device__ void flux_rusanov(double g, const double* L, const double* R, double nx, double ny, double nz, double* F) {
  const double ig1 = 1.0 / (g - 1.0);
  double vnl = L[2] * nx + L[3] * ny + L[4] * nz;
  double vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  double al = sqrt(g * L[1] / L[0]);
  double ar = sqrt(g * R[1] / R[0]);
  double ray = fmax(fabs(vnl) + al, fabs(vnr) + ar);
  double rel = ig1 * L[1] + 0.5 * L[0] * (L[2] * L[2] + L[3] * L[3] + L[4] * L[4]);
  double rer = ig1 * R[1] + 0.5 * R[0] * (R[2] * R[2] + R[3] * R[3] + R[4] * R[4]);
  F[0] = 0.5 * ((vnl + ray) * L[0] + (vnr - ray) * R[0]);
  F[1] = 0.5 * ((vnl + ray) * rel + (vnr - ray) * rer + vnl * L[1] + vnr * R[1]);
  double a = (vnl + ray) * L[0], b = (vnr - ray) * R[0], pp = L[1] + R[1];
  F[2] = 0.5 * ((a * L[2] + b * R[2]) + pp * nx);
  F[3] = 0.5 * ((a * L[3] + b * R[3]) + pp * ny);
  F[4] = 0.5 * ((a * L[4] + b * R[4]) + pp * nz);
}

// Roe flux-difference splitting with Harten's entropy fix (new: Typhon has no Roe flux)
__device__ void flux_roe(double g, double eps, const double* L, const double* R, double nx, double ny, double nz,
                         double* F) {
  const double ig1 = 1.0 / (g - 1.0);
  const double gig1 = g / (g - 1.0);
  double t1 = sqrt(R[0] / L[0]);
  double rroe = L[0] * t1;
  double kl = 1.0 / (1.0 + t1), kr = t1 * kl;
  double ux = kl * L[2] + kr * R[2], uy = kl * L[3] + kr * R[3], uz = kl * L[4] + kr * R[4];
  double sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4];
  double sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  double hl = gig1 * L[1] / L[0] + 0.5 * sqL;
  double hr = gig1 * R[1] / R[0] + 0.5 * sqR;
  double hroe = kl * hl + kr * hr;
  double q2 = ux * ux + uy * uy + uz * uz;
  double a2 = (g - 1.0) * (hroe - 0.5 * q2);
  double a = sqrt(a2);
  double vn = ux * nx + uy * ny + uz * nz;
  double vnl = L[2] * nx + L[3] * ny + L[4] * nz;
  double vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  double rel = ig1 * L[1] + 0.5 * L[0] * sqL;
  double rer = ig1 * R[1] + 0.5 * R[0] * sqR;
  double drho = R[0] - L[0], dp = R[1] - L[1], dvn = vnr - vnl;
  double dux = R[2] - L[2], duy = R[3] - L[3], duz = R[4] - L[4];
  double al1 = (dp - rroe * a * dvn) / (2.0 * a2);
  double al5 = (dp + rroe * a * dvn) / (2.0 * a2);
  double al2 = drho - dp / a2;
  double dutx = dux - dvn * nx, duty = duy - dvn * ny, dutz = duz - dvn * nz;
  double l1 = fabs(vn - a), l5 = fabs(vn + a), l2 = fabs(vn);
  double delta = eps * a;
  if (l1 < delta) l1 = (l1 * l1 + delta * delta) / (2.0 * delta);
  if (l5 < delta) l5 = (l5 * l5 + delta * delta) / (2.0 * delta);
  double w1 = l1 * al1, w2 = l2 * al2, w5 = l5 * al5, ws = l2 * rroe;
  double d_mass = w1 + w2 + w5;
  double dmx = w1 * (ux - a * nx) + w2 * ux + w5 * (ux + a * nx) + ws * dutx;
  double dmy = w1 * (uy - a * ny) + w2 * uy + w5 * (uy + a * ny) + ws * duty;
  double dmz = w1 * (uz - a * nz) + w2 * uz + w5 * (uz + a * nz) + ws * dutz;
  double d_ener = w1 * (hroe - a * vn) + w2 * (0.5 * q2) + w5 * (hroe + a * vn) +
                  ws * ((ux * dux + uy * duy + uz * duz) - vn * dvn);
  double ml = vnl * L[0], mr = vnr * R[0];
  F[0] = 0.5 * (ml + mr - d_mass);
  F[1] = 0.5 * (vnl * (rel + L[1]) + vnr * (rer + R[1]) - d_ener);
  F[2] = 0.5 * ((ml * L[2] + L[1] * nx) + (mr * R[2] + R[1] * nx) - dmx);
  F[3] = 0.5 * ((ml * L[3] + L[1] * ny) + (mr * R[3] + R[1] * ny) - dmy);
  F[4] = 0.5 * ((ml * L[4] + L[1] * nz) + (mr * R[4] + R[1] * nz) - dmz);
}

// ===========================================================================
// Fast mode.  Same mathematics, fewer FP64 operations: on GB300 the FP64 pipe (about 2
// DFMA per SM per clock, a division or square root costing about ten) bounds this path,
// so reciprocals, reconstruction weights and geometric factors are precomputed once
// (HBM-resident) and the per-stage work avoids divisions.

// Roe flux with shared reciprocals: no division, 1 reciprocal and 3 reciprocal square roots
// by Newton-Raphson steps (fastmath.cuh) per face.  The same flux as flux_roe, regrouped so
// that the central and dissipative parts share their products:
//   2 F_mass = m_L + m_R - d_mass                       (m = rho u.n)
//   2 F_ener = m_L H_L + m_R H_R - d_ener               (rho u.n (rho E + p) = m H)
//   2 F_mom  = A u_L + B u_R + c_n n, with the Roe velocity u~ = k_L u_L + k_R u_R and the
//              shear jump written through u_R - u_L:
//              A = m_L + ws - d_mass k_L, B = m_R - ws - d_mass k_R,
//              c_n = p_L + p_R - (w5 - w1) a + ws (u_R - u_L).n
__device__ void flux_roe_fast(const SpatOpts& o, const double* L, const double* R, double nx, double ny, double nz,
                              double S, double* F) {
  const double g1 = o.gamma - 1.0, eps = o.entropy_fix, ieps = o.inv_entropy_fix, gig1 = o.gig1;
  // Roe weights from one reciprocal square root: with y = 1/sqrt(rho_L rho_R),
  // rroe = sqrt(rho_L rho_R) = rho_L rho_R y, kl = sqrt(rho_L) / (sqrt(rho_L) + sqrt(rho_R)) =
  // rho_L / (rho_L + rroe), kr = rroe / (rho_L + rroe), 1/rho_L = y^2 rho_R, 1/rho_R = y^2 rho_L
  const double P = L[0] * R[0], y = rsqrt_nr(P), y2 = y * y;
  const double rroe = P * y;
  const double inv = rcp_nr(L[0] + rroe);
  const double kl = L[0] * inv, kr = rroe * inv;
  const double iL = y2 * R[0], iR = y2 * L[0];
  const double ux = kl * L[2] + kr * R[2], uy = kl * L[3] + kr * R[3], uz = kl * L[4] + kr * R[4];
  const double sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4];
  const double sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  const double hl = (gig1 * L[1]) * iL + 0.5 * sqL, hr = (gig1 * R[1]) * iR + 0.5 * sqR;
  const double hroe = kl * hl + kr * hr;
  const double q2 = ux * ux + uy * uy + uz * uz;
  const double a2 = g1 * (hroe - 0.5 * q2);
  const double ra = rsqrt_nr(a2), a = a2 * ra, ia2 = ra * ra;
  const double vn = ux * nx + uy * ny + uz * nz;
  const double vnl = L[2] * nx + L[3] * ny + L[4] * nz, vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  const double drho = R[0] - L[0], dp = R[1] - L[1], dvn = vnr - vnl;
  const double h = 0.5 * ia2, rad = rroe * a * dvn;
  const double al1 = (dp - rad) * h, al5 = (dp + rad) * h, al2 = drho - dp * ia2;
  double l1 = fabs(vn - a), l5 = fabs(vn + a);
  const double l2 = fabs(vn);
  const double delta = eps * a;
  // non-negative doubles compare like their bit patterns: test on the integer pipe
  if (__double_as_longlong(l1) < __double_as_longlong(delta) || __double_as_longlong(l5) < __double_as_longlong(delta)) {
    const double hd = 0.5 * ra * ieps;  // 1 / (2 delta)
    if (l1 < delta) l1 = (l1 * l1 + delta * delta) * hd;
    if (l5 < delta) l5 = (l5 * l5 + delta * delta) * hd;
  }
  const double w1 = l1 * al1, w2 = l2 * al2, w5 = l5 * al5, ws = l2 * rroe;
  const double d_mass = w1 + w2 + w5;
  const double wa = (w5 - w1) * a;
  const double ml = vnl * L[0], mr = vnr * R[0];
  const double hs = 0.5 * S;  // flux times surface: the 1/2 of the Roe average folded in
  // momentum
  const double A = ml + ws - d_mass * kl, B = mr - ws - d_mass * kr;
  const double cn = (L[1] + R[1]) - wa + ws * dvn;
  F[2] = hs * (A * L[2] + B * R[2] + cn * nx);
  F[3] = hs * (A * L[3] + B * R[3] + cn * ny);
  F[4] = hs * (A * L[4] + B * R[4] + cn * nz);
  // energy
  const double udu = ux * (R[2] - L[2]) + uy * (R[3] - L[3]) + uz * (R[4] - L[4]);
  const double d_ener = (w1 + w5) * hroe + wa * vn + w2 * (0.5 * q2) + ws * (udu - vn * dvn);
  F[1] = hs * (ml * hl + mr * hr - d_ener);
  F[0] = hs * (ml + mr - d_mass);
}

// HLLC (calc_flux_hllc.f90 with beta = 1) with shared reciprocals: no division; the
// reciprocals, square roots and reciprocal square roots by Newton-Raphson iterations
// (fastmath.cuh), the Roe weights and both 1/rho from one reciprocal square root.
__device__ void flux_hllc_fast(const SpatOpts& o, const double* L, const double* R, double nx, double ny, double nz,
                               double* F) {
  const double g = o.gamma, ig1 = o.ig1, gig1 = o.gig1;
  // Roe weights from one reciprocal square root (as flux_roe_fast)
  const double P = L[0] * R[0], y = rsqrt_nr(P), y2 = y * y;
  const double rroe = P * y;
  const double inv = rcp_nr(L[0] + rroe);
  const double kl = L[0] * inv, kr = rroe * inv;
  const double iL = y2 * R[0], iR = y2 * L[0];
  const double rux = kl * L[2] + kr * R[2], ruy = kl * L[3] + kr * R[3], ruz = kl * L[4] + kr * R[4];
  const double sqL = L[2] * L[2] + L[3] * L[3] + L[4] * L[4];
  const double sqR = R[2] * R[2] + R[3] * R[3] + R[4] * R[4];
  const double hroe = kl * (gig1 * L[1] * iL + 0.5 * sqL) + kr * (gig1 * R[1] * iR + 0.5 * sqR);
  const double vnl = L[2] * nx + L[3] * ny + L[4] * nz, vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  const double al = sqrt_nr(g * L[1] * iL), ar = sqrt_nr(g * R[1] * iR);
  const double vm = rux * nx + ruy * ny + ruz * nz;
  const double am = sqrt_nr((g - 1.0) * (hroe - 0.5 * (rux * rux + ruy * ruy + ruz * ruz)));
  const double rel = ig1 * L[1] + 0.5 * L[0] * sqL, rer = ig1 * R[1] + 0.5 * R[0] * sqR;
  double sl, sr;
  hll_speeds(o, vnl, vnr, al, ar, vm, am, sl, sr);
  if (sl >= 0.0) {
    const double m0 = vnl * L[0];
    F[0] = m0; F[1] = vnl * (rel + L[1]);
    F[2] = m0 * L[2] + L[1] * nx; F[3] = m0 * L[3] + L[1] * ny; F[4] = m0 * L[4] + L[1] * nz;
  } else if (sr <= 0.0) {
    const double m0 = vnr * R[0];
    F[0] = m0; F[1] = vnr * (rer + R[1]);
    F[2] = m0 * R[2] + R[1] * nx; F[3] = m0 * R[3] + R[1] * ny; F[4] = m0 * R[4] + R[1] * nz;
  } else {
    const double rqL = L[0] * (sl - vnl), rqR = R[0] * (sr - vnr);
    const double Sst = (rqR * vnr - rqL * vnl - R[1] + L[1]) * rcp_nr(rqR - rqL);
    const bool left = Sst >= 0.0;
    const double* Q = left ? L : R;
    const double rq = left ? rqL : rqR, s = left ? sl : sr, vnq = left ? vnl : vnr, re = left ? rel : rer;
    const double iks = rcp_nr(s - Sst);
    const double pst = Q[1] - rq * (vnq - Sst);
    const double dp = pst - Q[1];
    const double m0 = Sst * iks;
    F[0] = m0 * rq;
    F[1] = Sst * (iks * (re * (s - vnq) - Q[1] * vnq + pst * Sst) + pst);
    F[2] = m0 * (rq * Q[2] + dp * nx) + pst * nx;
    F[3] = m0 * (rq * Q[3] + dp * ny) + pst * ny;
    F[4] = m0 * (rq * Q[4] + dp * nz) + pst * nz;
  }
}

// Laminar viscous flux added to F (per unit area), calc_flux_viscous_cell.f90:71-144, on the
// cell states and cell gradients of the face's two cells (integration_ns_ust.f90:139-159).
// Face gradients: CELL-AVERAGE a.grad_R + b.grad_L, or FULL with the compact correction along
// C_L C_R (interpface_gradient_vect.f90:59-81, interpface_gradn_scal.f90:60-90, theta = 1).
// On adiabatic-wall faces the conduction term is added back (ns_bocoflux.f90:60-108).
__device__ void add_viscous(const DevMesh& m, const DevState& s, const SpatOpts& o, int f, double* F) {
  const size_t ld = m.ldc, lf = m.ldf;
  const int icl = m.fc1[f], icr = m.fc2[f];
  const double* __restrict__ q = s.prim;
  const double* __restrict__ gr = s.grad;
  const double r = o.rgas;
  const double cp = o.gamma * r / (o.gamma - 1.0);
  const double dHL = m.vgeo[f], dHR = m.vgeo[lf + f];
  const double wx = m.vgeo[2 * lf + f], wy = m.vgeo[3 * lf + f], wz = m.vgeo[4 * lf + f];
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  const double vL[3] = {q[2 * ld + icl], q[3 * ld + icl], q[4 * ld + icl]};
  const double vR[3] = {q[2 * ld + icr], q[3 * ld + icr], q[4 * ld + icr]};
  double velH[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) velH[i] = dHR * vL[i] + dHL * vR[i];
  const double rL = q[icl], rR = q[icr], pL = q[ld + icl], pR = q[ld + icr];
  const double TL = pL / (rL * r), TR = pR / (rR * r);
  const double TH = dHR * TL + dHL * TR;
  const double rhoH = dHR * rL + dHL * rR;
  const double aL = 1.0 / (rL * r), bL = pL / ((rL * rL) * r);
  const double aR = 1.0 / (rR * r), bR = pR / ((rR * rR) * r);
  double gT[3];  // dHL gradT_R + dHR gradT_L
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double gTL = aL * gr[(3 + k) * ld + icl] - bL * gr[k * ld + icl];
    const double gTR = aR * gr[(3 + k) * ld + icr] - bR * gr[k * ld + icr];
    gT[k] = dHL * gTR + dHR * gTL;
  }
  const double mu = viscosity(o, rhoH, TH);
  double G[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      G[i][j] = dHL * gr[(6 + 3 * i + j) * ld + icr] + dHR * gr[(6 + 3 * i + j) * ld + icl];
  double gTH;
  if (o.viscous == TY_VISC_CELLFULL) {
    const double dLR2 = wx * wx + wy * wy + wz * wz;
    const double it = 1.0 / dLR2;
    const double ex = it * wx, ey = it * wy, ez = it * wz;
    double Fav[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) Fav[i] = vR[i] - vL[i] - (G[i][0] * wx + G[i][1] * wy + G[i][2] * wz);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      G[i][0] = G[i][0] + Fav[i] * ex;
      G[i][1] = G[i][1] + Fav[i] * ey;
      G[i][2] = G[i][2] + Fav[i] * ez;
    }
    const double pscal = (wx * nx + wy * ny + wz * nz) / dLR2;
    const double Fcomp = pscal * (TR - TL);
    const double tp = 1.0 * pscal;
    const double vix = nx - tp * wx, viy = ny - tp * wy, viz = nz - tp * wz;
    gTH = 1.0 * Fcomp + (gT[0] * vix + gT[1] * viy + gT[2] * viz);
  } else {
    gTH = gT[0] * nx + gT[1] * ny + gT[2] * nz;
  }
  double Sg[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Sg[i][j] = G[i][j] + G[j][i];
  const double addvisc = -(2.0 / 3.0) * (G[0][0] + G[1][1] + G[2][2]);
#pragma unroll
  for (int i = 0; i < 3; ++i) Sg[i][i] = Sg[i][i] + addvisc;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Sg[i][j] = mu * Sg[i][j];
  const double snx = Sg[0][0] * nx + Sg[0][1] * ny + Sg[0][2] * nz;
  const double sny = Sg[1][0] * nx + Sg[1][1] * ny + Sg[1][2] * nz;
  const double snz = Sg[2][0] * nx + Sg[2][1] * ny + Sg[2][2] * nz;
  const double svn = snx * velH[0] + sny * velH[1] + snz * velH[2];
  F[2] = F[2] - snx;
  F[3] = F[3] - sny;
  F[4] = F[4] - snz;
  F[1] = F[1] - svn;
  const double conduct = mu * cp / o.prandtl;
  F[1] = F[1] - conduct * gTH;
  if (f >= m.nfi && (m.fbc[f] == TY_BC_WALL || m.fbc[f] == TY_BC_NOSLIP)) F[1] = F[1] + conduct * gTH + 0.0;
}

__device__ __forceinline__ void face_flux_fast(const DevMesh& m, const DevState& s, const SpatOpts& o, int f,
                                               const double* QL, const double* QR, double* __restrict__ flux) {
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  double F[5];
  const double S = m.fs[f];
  if (o.scheme == TY_SCH_ROE && o.viscous == TY_VISC_NONE) {
    flux_roe_fast(o, QL, QR, nx, ny, nz, S, F);
  } else {
    if (o.scheme == TY_SCH_ROE) flux_roe_fast(o, QL, QR, nx, ny, nz, 1.0, F);
    else if (o.hll_family == 1) flux_hllc_fast(o, QL, QR, nx, ny, nz, F);
    else if (o.hll_family == 2) flux_hlle(o, QL, QR, nx, ny, nz, F);
    else if (o.scheme == TY_SCH_AUSMM) flux_ausmm(o.gamma, QL, QR, nx, ny, nz, F);
    else flux_rusanov(o.gamma, QL, QR, nx, ny, nz, F);
    if (o.viscous != TY_VISC_NONE) add_viscous(m, s, o, f, F);
#pragma unroll
    for (int v = 0; v < 5; ++v) F[v] = S * F[v];
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) flux[v * (size_t)m.ldf + f] = F[v];
}


__device__ __forceinline__ void face_flux(const DevMesh& m, const DevState& s, const SpatOpts& o, int f,
                                          const double* QL, const double* QR, double* __restrict__ flux) {
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  double F[5];
  if constexpr (kFast) {
    if (o.hll_family == 1) flux_hllc_fast(o, QL, QR, nx, ny, nz, F);
    else if (o.scheme == TY_SCH_RUSANOV) flux_rusanov(o.gamma, QL, QR, nx, ny, nz, F);
    else if (o.hll_family == 2) flux_hlle(o, QL, QR, nx, ny, nz, F);
    else if (o.scheme == TY_SCH_AUSMM) flux_ausmm(o.gamma, QL, QR, nx, ny, nz, F);
    else flux_roe_fast(o, QL, QR, nx, ny, nz, 1.0, F);  // unit surface
  } else {
    if (o.hll_family == 1) flux_hllc(o, QL, QR, nx, ny, nz, F);
    else if (o.scheme == TY_SCH_RUSANOV) flux_rusanov(o.gamma, QL, QR, nx, ny, nz, F);
    else if (o.hll_family == 2) flux_hlle(o, QL, QR, nx, ny, nz, F);
    else if (o.scheme == TY_SCH_AUSMM) flux_ausmm(o.gamma, QL, QR, nx, ny, nz, F);
    else flux_roe(o.gamma, o.entropy_fix, QL, QR, nx, ny, nz, F);
  }
  if (o.viscous != TY_VISC_NONE) add_viscous(m, s, o, f, F);
  const double S = m.fs[f];
#pragma unroll
  for (int v = 0; v < 5; ++v) flux[v * (size_t)m.ldf + f] = S * F[v];
}

// fused face states + flux (no post-limiter)
__global__ void __launch_bounds__(kBlock) k_face_flux(DevMesh m, DevState s, SpatOpts o) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  double QL[5], QR[5];
  recon(m, s, o, f, 0, QL);
  const int kind = f < m.nfi ? TY_BC_INTERIOR : m.fbc[f];
  if (kind == TY_BC_PERIODIC) {
    recon(m, s, o, m.part[f], 0, QR);  // cell_r(face) = cell_l(partner face)
    rot_to_face(m, f, QR);
  } else if (kind == TY_BC_WALL || kind == TY_BC_NOSLIP) {
    wall_state(m, f, QL, QR);
  } else if (kind == TY_BC_FARFIELD) {
    farfield_state(o, d3(m.fn, m.ldf, f, 0), d3(m.fn, m.ldf, f, 1), d3(m.fn, m.ldf, f, 2), QL, QR);
  } else if (kind >= TY_BC_INLET_SUB) {
    inout_state(m, o, f, kind, QL, QR);
  } else if (kind == TY_BC_SYMMETRY) {
#pragma unroll
    for (int v = 0; v < 5; ++v) QR[v] = QL[v];
    mirror(m, f, QR);
  } else {
    recon(m, s, o, f, 1, QR);
  }
  face_flux(m, s, o, f, QL, QR, s.flux);
}

// post-limiter path, 1: unlimited face states
__global__ void __launch_bounds__(kBlock) k_face_states(DevMesh m, DevState s, SpatOpts o) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  double Q[5];
  recon(m, s, o, f, 0, Q);
#pragma unroll
  for (int v = 0; v < 5; ++v) s.cl[v * (size_t)m.ldf + f] = Q[v];
  recon(m, s, o, f, 1, Q);
#pragma unroll
  for (int v = 0; v < 5; ++v) s.cr[v * (size_t)m.ldf + f] = Q[v];
}

// post-limiter path, 2: Barth-type ratio of each interior cell (postlimit_barth.f90:60-80,
// 140-170).  A face whose increment is exactly zero imposes no constraint.
__global__ void __launch_bounds__(kBlock) k_barth(DevMesh m, DevState s, double klim) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t ld = m.ldc, lf = m.ldf;
  double r[3] = {1.0, 1.0, 1.0};
  double qc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) qc[v] = s.prim[v * ld + c];
  for (int sl = 0; sl < m.nslot; ++sl) {
    int e = m.cf[sl * (size_t)m.nci + c];
    if (e < 0) break;
    int f = e >> 1, side = e & 1;
    int nb = side ? m.fc1[f] : m.fc2[f];
    const double* qf = side ? s.cr : s.cl;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double LR = s.prim[v * ld + nb] - qc[v];  // = +-(q(fc2) - q(fc1)) seen from c
      double den = qf[v * lf + f] - qc[v];
      if (den != 0.0) {
        double l = fmax(klim * (LR / den), 0.0);
        int k = v < 2 ? v : 2;
        r[k] = fmin(r[k], l);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) s.ratio[k * ld + c] = r[k];
}

// post-limiter path, 3: limited states + flux
__global__ void __launch_bounds__(kBlock) k_face_flux_lim(DevMesh m, DevState s, SpatOpts o) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const size_t ld = m.ldc, lf = m.ldf;
  double QL[5], QR[5];
  auto limited = [&](int face, int side, double* Q) {
    int c = side ? m.fc2[face] : m.fc1[face];
    const double* qf = side ? s.cr : s.cl;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double qc = s.prim[v * ld + c];
      double rr = s.ratio[(v < 2 ? v : 2) * ld + c];
      Q[v] = qc + rr * (qf[v * lf + face] - qc);
    }
  };
  limited(f, 0, QL);
  const int kind = f < m.nfi ? TY_BC_INTERIOR : m.fbc[f];
  if (kind == TY_BC_PERIODIC) {
    limited(m.part[f], 0, QR);
    rot_to_face(m, f, QR);
  } else if (kind == TY_BC_WALL || kind == TY_BC_NOSLIP) {
    wall_state(m, f, QL, QR);
  } else if (kind == TY_BC_FARFIELD) {
    farfield_state(o, d3(m.fn, m.ldf, f, 0), d3(m.fn, m.ldf, f, 1), d3(m.fn, m.ldf, f, 2), QL, QR);
  } else if (kind >= TY_BC_INLET_SUB) {
    inout_state(m, o, f, kind, QL, QR);
  } else if (kind == TY_BC_SYMMETRY) {
#pragma unroll
    for (int v = 0; v < 5; ++v) QR[v] = QL[v];
    mirror(m, f, QR);
  } else {
    limited(f, 1, QR);
  }
  face_flux(m, s, o, f, QL, QR, s.flux);
}


// Increment q_face - q_c of the 5 primitive variables on one side of face f, from the
// cell's gradient gr (15), its value qc and dq = q_nb - q_c.
__device__ __forceinline__ void delta_fast(const DevMesh& m, const SpatOpts& o, int f, int side, const double* gr,
                                           const double* dq, double* D) {
  const size_t lf = m.ldf;
  if ((o.highres == TY_HRES_MUSCL || o.highres == TY_HRES_MUSCLUNS) && o.limiter == TY_LIM_NONE) {
    const double wx = m.recw[(4 * side) * lf + f], wy = m.recw[(4 * side + 1) * lf + f];
    const double wz = m.recw[(4 * side + 2) * lf + f], k = m.recw[(4 * side + 3) * lf + f];
#pragma unroll
    for (int v = 0; v < 5; ++v) D[v] = fma(gr[3 * v], wx, fma(gr[3 * v + 1], wy, fma(gr[3 * v + 2], wz, dq[v] * k)));
    return;
  }
  const double ux = d3(m.uLR, m.ldf, f, 0), uy = d3(m.uLR, m.ldf, f, 1), uz = d3(m.uLR, m.ldf, f, 2);
  const double idLR = m.invdLR[f];
  const double sgn = side ? -1.0 : 1.0;  // (q(fc2) - q(fc1)) = sgn * dq
  if (o.highres == TY_HRES_MUSCLFAST) {
    const double k = side ? m.kRF[f] : m.kLF[f];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double LR = sgn * dq[v] * idLR;
      double sg = LR;
      if (o.limiter != TY_LIM_NONE) {
        const double g = gr[3 * v] * ux + gr[3 * v + 1] * uy + gr[3 * v + 2] * uz;
        sg = apply_lim(o.limiter, false, v < 2, g, LR);
      }
      D[v] = sg * k;
    }
    return;
  }
  const bool uns = o.highres == TY_HRES_MUSCLUNS;
  const double* CF = side ? m.RF : m.LF;
  const double cx = d3(CF, m.ldf, f, 0), cy = d3(CF, m.ldf, f, 1), cz = d3(CF, m.ldf, f, 2);
  const double uc = ux * cx + uy * cy + uz * cz;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double LR = sgn * dq[v] * idLR;
    const double g = gr[3 * v] * ux + gr[3 * v + 1] * uy + gr[3 * v + 2] * uz;
    const double sg = (o.limiter == TY_LIM_NONE ? LR : apply_lim(o.limiter, uns, v < 2, g, LR)) - g;
    D[v] = gr[3 * v] * cx + gr[3 * v + 1] * cy + gr[3 * v + 2] * cz + sg * uc;
  }
}

// Fused per-cell kernel: least-squares gradient (A^-1 d weights), face increments on every
// face of the cell, Barth-type ratio without per-face divisions, and the limited face
// states written once per face side (cl for the fc1 side, cr for the fc2 side).
// The neighbour differences dq of the gradient pass and the increments are staged in shared
// memory ([slot*5+var][thread], conflict-free), so each is computed once and the kernel keeps
// few registers live (four blocks of 128 threads per SM).
// The ratio min_f max(klim (q_nb - q_c)/increment, 0) is tracked as a fraction n/d; the
// comparisons run on the integer pipe (positive finite doubles order like their bit
// patterns), leaving the FP64 pipe to the arithmetic, and the one division per variable
// group is a Newton-Raphson reciprocal.  The increment is the reconstruction's value (the
// exact mode, like Typhon, rounds it through the face value first); an increment of exactly
// zero imposes no constraint in both modes.
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }

//
// With DevMesh::mtab (MUSCL / MUSCL-UNS without limiter) the increments come from the cell's
// matrix, D_i = sum_j M_ij dq_j: the gradient G = sum_j (+-A^-1 d_j) dq_j and the increment
// D_i = G . w_i + dq_i k_i folded into one product of nslot^2 multiply-adds per variable (16
// for a tetrahedron, against 12 for the gradient and 16 for the increments), read coalesced
// per cell instead of per face; the gradient itself is then computed only when asked
// (want_grad: a viscous flux or the adjoint reads it).
template <int NS, int BLK>
__global__ void __launch_bounds__(BLK, 512 / BLK) k_cell_fast(DevMesh m, DevState s, SpatOpts o, double klim,
                                                              bool want_grad) {
  __shared__ double sD[NS * 5][BLK];
  __shared__ double sQ[NS * 5][BLK];
  const int c = blockIdx.x * BLK + threadIdx.x;
  if (c >= m.nci) return;
  const int t = threadIdx.x;
  const size_t ld = m.ldc, lf = m.ldf, ni = m.nci;
  const double* __restrict__ prim = s.prim;
  double qc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) qc[v] = prim[v * ld + c];
  const bool mt = m.mtab != nullptr;
  const bool grad = !mt || want_grad;
  double gr[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) gr[k] = 0.0;
  // the gather-list entries and neighbours of every slot first, so that the neighbour loads
  // below are independent of each other and issue together
  int es[NS], nbs[NS];
  int ns = 0;
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    es[sl] = sl < m.nslot ? m.cf[sl * ni + c] : -1;
    nbs[sl] = es[sl] >= 0 ? m.cfn[sl * ni + c] : c;
    ns += es[sl] >= 0 ? 1 : 0;
  }
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int e = es[sl];
    if (e < 0) continue;
    const int f = e >> 1, side = e & 1, nb = nbs[sl];
    if (grad) {
      // q(fc2) - q(fc1) = +-dq: the weight's sign flipped on the integer pipe for side 1
      const long long sb = (long long)side << 63;
      const double wx = __longlong_as_double(__double_as_longlong(m.lsqw[(3 * side) * lf + f]) ^ sb);
      const double wy = __longlong_as_double(__double_as_longlong(m.lsqw[(3 * side + 1) * lf + f]) ^ sb);
      const double wz = __longlong_as_double(__double_as_longlong(m.lsqw[(3 * side + 2) * lf + f]) ^ sb);
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double dq = prim[v * ld + nb] - qc[v];
        sQ[sl * 5 + v][t] = dq;
        gr[3 * v] = fma(dq, wx, gr[3 * v]);
        gr[3 * v + 1] = fma(dq, wy, gr[3 * v + 1]);
        gr[3 * v + 2] = fma(dq, wz, gr[3 * v + 2]);
      }
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) sQ[sl * 5 + v][t] = prim[v * ld + nb] - qc[v];
    }
  }
  if (grad) {
#pragma unroll
    for (int k = 0; k < 15; ++k) s.grad[k * ld + c] = gr[k];
  }
  const bool barth = o.postlim != TY_POSTLIM_NONE;
  double bn[3] = {1.0, 1.0, 1.0}, bd[3] = {klim, klim, klim};
  bool zero[3] = {false, false, false};
  for (int sl = 0; sl < ns; ++sl) {
    const int e = m.cf[sl * ni + c], f = e >> 1, side = e & 1;
    double dq[5], D[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) dq[v] = sQ[sl * 5 + v][t];
    if (mt) {
      // the row's NS coefficients loaded together (one memory latency per row, not per term)
      const double* M = m.mtab + (size_t)sl * m.nslot * ni + c;
      double mr[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) mr[j] = j < ns ? __ldg(M + (size_t)j * ni) : 0.0;
#pragma unroll
      for (int v = 0; v < 5; ++v) D[v] = 0.0;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        if (j < ns) {
#pragma unroll
          for (int v = 0; v < 5; ++v) D[v] = fma(mr[j], sQ[j * 5 + v][t], D[v]);
        }
      }
    } else {
      delta_fast(m, o, f, side, gr, dq, D);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double den = D[v];
      sD[sl * 5 + v][t] = den;
      if (barth) {
        const int k = v < 2 ? v : 2;
        const long long bden = dbits(den), bdq = dbits(dq[v]);
        if ((bden << 1) != 0) {                                   // den != 0
          if ((bdq << 1) == 0 || ((bdq ^ bden) < 0)) {             // dq/den <= 0
            zero[k] = true;
          } else {
            const double x = fabs(dq[v]) * bd[k], y = bn[k] * fabs(den);
            if (dbits(x) < dbits(y)) { bn[k] = fabs(dq[v]); bd[k] = fabs(den); }
          }
        }
      }
    }
  }
  double r[3] = {1.0, 1.0, 1.0};
  if (barth) {
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = zero[k] ? 0.0 : fmin(1.0, klim * bn[k] * rcp_nr(bd[k]));
#pragma unroll
    for (int k = 0; k < 3; ++k) s.ratio[k * ld + c] = r[k];
  }
  for (int sl = 0; sl < ns; ++sl) {
    const int e = m.cf[sl * ni + c], f = e >> 1, side = e & 1;
    double* out = side ? s.cr : s.cl;
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * lf + f] = fma(r[v < 2 ? v : 2], sD[sl * 5 + v][t], qc[v]);
  }
}

// k_cell_fast for the case of DevMesh::mtab without a gradient output (MUSCL / MUSCL-UNS
// without limiter, inviscid): the neighbour differences and the increments of the (at most
// NS) faces stay in registers instead of shared memory, which the FP64 pipe no longer waits
// for.  Same arithmetic as k_cell_fast.
template <int NS, int BLK>
__global__ void __launch_bounds__(BLK, 512 / BLK) k_cell_fast_mt(DevMesh m, DevState s, SpatOpts o, double klim) {
  const int c = blockIdx.x * BLK + threadIdx.x;
  if (c >= m.nci) return;
  const size_t ld = m.ldc, lf = m.ldf, ni = m.nci;
  const double* __restrict__ prim = s.prim;
  int es[NS], nbs[NS];
  int ns = 0;
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    es[sl] = sl < m.nslot ? m.cf[sl * ni + c] : -1;
    nbs[sl] = es[sl] >= 0 ? m.cfn[sl * ni + c] : c;
    ns += es[sl] >= 0 ? 1 : 0;
  }
  double qc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) qc[v] = prim[v * ld + c];
  double dq[NS][5];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl)
#pragma unroll
    for (int v = 0; v < 5; ++v) dq[sl][v] = prim[v * ld + nbs[sl]] - qc[v];  // 0 on an unused slot
  const bool barth = o.postlim != TY_POSTLIM_NONE;
  double bn[3] = {1.0, 1.0, 1.0}, bd[3] = {klim, klim, klim};
  bool zero[3] = {false, false, false};
  double D[NS][5];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const double* M = m.mtab + (size_t)sl * m.nslot * ni + c;
    double mr[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) mr[j] = (sl < ns && j < ns) ? __ldg(M + (size_t)j * ni) : 0.0;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double d = 0.0;
#pragma unroll
      for (int j = 0; j < NS; ++j) d = fma(mr[j], dq[j][v], d);
      D[sl][v] = d;
      if (barth && sl < ns) {
        const int k = v < 2 ? v : 2;
        const long long bden = dbits(d), bdq = dbits(dq[sl][v]);
        if ((bden << 1) != 0) {                                   // d != 0
          if ((bdq << 1) == 0 || ((bdq ^ bden) < 0)) {             // dq/d <= 0
            zero[k] = true;
          } else {
            const double x = fabs(dq[sl][v]) * bd[k], y = bn[k] * fabs(d);
            if (dbits(x) < dbits(y)) { bn[k] = fabs(dq[sl][v]); bd[k] = fabs(d); }
          }
        }
      }
    }
  }
  double r[3] = {1.0, 1.0, 1.0};
  if (barth) {
#pragma unroll
    for (int k = 0; k < 3; ++k) r[k] = zero[k] ? 0.0 : fmin(1.0, klim * bn[k] * rcp_nr(bd[k]));
#pragma unroll
    for (int k = 0; k < 3; ++k) s.ratio[k * ld + c] = r[k];
  }
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    if (sl >= ns) continue;
    const int e = es[sl], f = e >> 1, side = e & 1;
    double* out = side ? s.cr : s.cl;
#pragma unroll
    for (int v = 0; v < 5; ++v) out[v * lf + f] = fma(r[v < 2 ? v : 2], D[sl][v], qc[v]);
  }
}

#if TY_FAST
// DevMesh::mtab of every interior cell: M_ij = (+-A^-1 d_j) . w_i + k_i [i == j] over the
// cell's gather-list faces i, j (w, k: the reconstruction weights recw of face i on the cell's
// side; the least-squares weight's sign flipped for the fc2 side, as k_cell_fast does);
// zero outside the cell's faces
__global__ void k_build_mtab(DevMesh m, double* __restrict__ mt) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t n = m.nci, lf = m.ldf;
  const int ns = m.nslot;
  for (int i = 0; i < ns; ++i) {
    const int ei = m.cf[i * n + c];
    for (int j = 0; j < ns; ++j) {
      const int ej = m.cf[j * n + c];
      double v = 0.0;
      if (ei >= 0 && ej >= 0) {
        const int fi = ei >> 1, si = ei & 1, fj = ej >> 1, sj = ej & 1;
        const double sg = sj ? -1.0 : 1.0;
        for (int k = 0; k < 3; ++k) v += sg * m.lsqw[(3 * sj + k) * lf + fj] * m.recw[(4 * si + k) * lf + fi];
        if (i == j) v += m.recw[(4 * si + 3) * lf + fi];
      }
      mt[((size_t)i * ns + j) * n + c] = v;
    }
  }
}

cudaError_t build_mtab(const DevMesh& m, double* mtab, cudaStream_t st) {
  k_build_mtab<<<(unsigned)((m.nci + kBlock - 1) / kBlock), kBlock, 0, st>>>(m, mtab);
  return cudaGetLastError();
}
#endif

// face fluxes from the limited states of k_cell_fast
__global__ void __launch_bounds__(kBlock) k_face_flux_fast(DevMesh m, DevState s, SpatOpts o) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const size_t lf = m.ldf;
  double QL[5], QR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) QL[v] = s.cl[v * lf + f];
  const int kind = f < m.nfi ? TY_BC_INTERIOR : m.fbc[f];
  if (kind == TY_BC_PERIODIC) {
    const int p = m.part[f];
#pragma unroll
    for (int v = 0; v < 5; ++v) QR[v] = s.cl[v * lf + p];
    rot_to_face(m, f, QR);
  } else if (kind == TY_BC_WALL || kind == TY_BC_NOSLIP) {
    wall_state(m, f, QL, QR);
  } else if (kind == TY_BC_FARFIELD) {
    farfield_state(o, d3(m.fn, m.ldf, f, 0), d3(m.fn, m.ldf, f, 1), d3(m.fn, m.ldf, f, 2), QL, QR);
  } else if (kind >= TY_BC_INLET_SUB) {
    inout_state(m, o, f, kind, QL, QR);
  } else if (kind == TY_BC_SYMMETRY) {
#pragma unroll
    for (int v = 0; v < 5; ++v) QR[v] = QL[v];
    mirror(m, f, QR);
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) QR[v] = s.cr[v * lf + f];
  }
  face_flux_fast(m, s, o, f, QL, QR, s.flux);
}

// ---------------------------------------------------------------------------
// residual R_c = dt/V_c * sum(+-F S), in the colour order of flux_to_res
__device__ __forceinline__ void gather_residual(const DevMesh& m, const DevState& s, int c, double R[5]) {
#pragma unroll
  for (int v = 0; v < 5; ++v) R[v] = 0.0;
  const double* __restrict__ F = s.flux;
  const size_t lf = m.ldf;
  for (int sl = 0; sl < m.nslot; ++sl) {
    int e = m.cf[sl * (size_t)m.nci + c];
    if (e < 0) break;
    int f = e >> 1;
    if (e & 1) {
#pragma unroll
      for (int v = 0; v < 5; ++v) R[v] = R[v] + F[v * lf + f];
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) R[v] = R[v] - F[v * lf + f];
    }
  }
}

__device__ __forceinline__ double load_dt(double dt, const unsigned long long* dtbits) {
  return dtbits ? __longlong_as_double((long long)*dtbits) : dt;
}

__global__ void __launch_bounds__(kBlock) k_gather(DevMesh m, DevState s, double dt, const unsigned long long* dtbits) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  double R[5];
  gather_residual(m, s, c, R);
  const double coef = load_dt(dt, dtbits) / m.cvol[c];
#pragma unroll
  for (int v = 0; v < 5; ++v) s.res[v * (size_t)m.ldc + c] = coef * R[v];
}

// per-cell stability time step; returns false for negative or NaN internal energy
__device__ __forceinline__ bool cell_dt(const DevMesh& m, double gamma, double cfl, int c, const double u[5], double& dt) {
  const double gg1 = gamma * (gamma - 1.0);
  double d;
  if constexpr (kFast) d = cfl * m.geo2[c];
  else d = cfl * 2.0 * m.cvol[c] / m.sumS[c];
  if constexpr (kFast) {
    const double irho = rcp_nr(u[0]);
    const double rv2 = u[2] * u[2] + u[3] * u[3] + u[4] * u[4];
    const double a2 = (u[1] - 0.5 * rv2 * irho) * gg1 * irho;
    if (!(a2 > 0.0)) return false;
    dt = d * rcp_nr(sqrt_nr(rv2) * irho + sqrt_nr(a2));
    return true;
  }
  double irho = 1.0 / u[0];
  double rv2 = u[2] * u[2] + u[3] * u[3] + u[4] * u[4];
  double a2 = (u[1] - 0.5 * rv2 * irho) * gg1 * irho;
  if (!(a2 > 0.0)) return false;
  dt = d / (sqrt(rv2) * irho + sqrt(a2));
  return true;
}

// block minimum of positive doubles through their bit patterns (order-independent, exact)
__device__ __forceinline__ void block_min_dt(double dt, unsigned long long* dtbits) {
  __shared__ unsigned long long smin[kBlock / 32];
  unsigned long long b = (unsigned long long)__double_as_longlong(dt);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
    b = t < b ? t : b;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) smin[w] = b;
  __syncthreads();
  if (w == 0) {
    b = lane < (int)(blockDim.x >> 5) ? smin[lane] : ~0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
      b = t < b ? t : b;
    }
    if (lane == 0) atomicMin(dtbits, b);
  }
}

__device__ __forceinline__ void flag_error(int* err, int code, int cell) {
  if (atomicCAS(err, 0, code) == 0) err[1] = cell;
}

__global__ void __launch_bounds__(kBlock) k_timestep(DevMesh m, const double* __restrict__ cons, double gamma,
                                                      double cfl, unsigned long long* dtbits, int* err) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  double dt = __longlong_as_double(0x7fefffffffffffffll);  // largest finite double
  if (c < m.nci) {
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = cons[v * (size_t)m.ldc + c];
    double d;
    if (cell_dt(m, gamma, cfl, c, u, d)) {
      dt = d;
      if (!(d > 0.0)) flag_error(err, TY_ERR_NANDT, c);
    } else {
      flag_error(err, TY_ERR_NEGENERGY, c);
    }
  }
  block_min_dt(dt, dtbits);
}

// Runge-Kutta update at the end of a stage.  Applies the plan's partial sums, the final
// combination, and derives the primitive variables of the new state (and its time step
// after the last stage when dtbits_next is given).
__global__ void __launch_bounds__(kBlock) k_rk_update(DevMesh m, DevState s, RkStagePlan plan, double gamma, double dt,
                                                       const unsigned long long* dtbits, unsigned long long* dtbits_next,
                                                       double cfl) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = c < m.nci;
  double dtc = __longlong_as_double(0x7fefffffffffffffll);
  if (active) {
    const size_t ld = m.ldc;
    double R[5];
    gather_residual(m, s, c, R);
    const double dtv = plan.dtloc ? plan.dtloc[c] : load_dt(dt, dtbits);
    // exact: R = (dt/V) R first, as flux_to_res does; fast: dt/V folded into each stage
    // coefficient (one product per coefficient instead of one per variable)
    double coef, rs = 1.0;
    if constexpr (kFast) {
      rs = dtv * m.invV[c];
    } else {
      coef = dtv / m.cvol[c];
#pragma unroll
      for (int v = 0; v < 5; ++v) R[v] = coef * R[v];
    }
    double u0[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u0[v] = s.u0[v * ld + c];
    double next[5];
    bool have_next = false;
    for (int k = 0; k < plan.nops; ++k) {
      const RkOp op = plan.ops[k];
      double* part = s.pk[op.target];
      const double oc = kFast ? op.c * rs : op.c;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double base = op.from_u0 ? u0[v] : part[v * ld + c];
        double val = base + oc * R[v];
        if (op.is_next) next[v] = val;
        else part[v * ld + c] = val;
      }
      if (op.is_next) have_next = true;
    }
    if (plan.has_acc) {
      const double ca = kFast ? plan.c_acc * rs : plan.c_acc;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double a = plan.acc_init ? ca * R[v] : s.acc[v * ld + c] + ca * R[v];
        if (plan.final_stage) next[v] = u0[v] + a;
        if (!plan.final_stage || plan.store_acc) s.acc[v * ld + c] = a;
      }
      if (plan.final_stage) have_next = true;
    }
    if (have_next) {
      double* dst = plan.final_stage ? s.u0 : s.cur;
#pragma unroll
      for (int v = 0; v < 5; ++v) dst[v * ld + c] = next[v];
      double q[5];
      cons_to_prim(gamma, next, q);
#pragma unroll
      for (int v = 0; v < 5; ++v) s.prim[v * ld + c] = q[v];
      if (dtbits_next) {
        double d;
        if (cell_dt(m, gamma, cfl, c, next, d)) {
          dtc = d;
          if (!(d > 0.0)) flag_error(s.err, TY_ERR_NANDT, c);
        } else {
          flag_error(s.err, TY_ERR_NEGENERGY, c);
        }
      }
    }
  }
  if (dtbits_next) block_min_dt(dtc, dtbits_next);
}

// ---------------------------------------------------------------------------
// launch sequences
inline unsigned nblk(int n) { return (unsigned)((n + kBlock - 1) / kBlock); }

cudaError_t prim_from(const DevMesh& m, const DevState& s, const SpatOpts& o, const double* cons,
                      cudaStream_t st, Prof* pr) {
  if (m.nci > 0)
    pr->launch(K_PRIM, st, [&] { k_prim<<<nblk(m.nci), kBlock, 0, st>>>(m, cons, s.prim, o.gamma); });
  return cudaGetLastError();
}

// everything between the primitive variables of a stage state and the face fluxes
cudaError_t residual_faces(const DevMesh& m, const DevState& s, const SpatOpts& o, cudaStream_t st, Prof* pr) {
  if (m.ng > 0)
    pr->launch(K_GHOST_PRIM, st, [&] { k_ghost_prim<<<nblk(m.ng), kBlock, 0, st>>>(m, s.prim, o); });
  if (kFast && o.highres != TY_HRES_NONE) {
    const double klim = o.postlim == TY_POSTLIM_SUPERBARTH ? 1.0 : 0.5;
    if (m.nslot <= 4 && m.mtab && o.viscous == TY_VISC_NONE)
      pr->launch(K_CELL_FAST, st, [&] {
        k_cell_fast_mt<4, 128><<<(unsigned)((m.nci + 127) / 128), 128, 0, st>>>(m, s, o, klim);
      });
    else if (m.nslot <= 4)
      pr->launch(K_CELL_FAST, st, [&] {
        k_cell_fast<4, 128><<<(unsigned)((m.nci + 127) / 128), 128, 0, st>>>(m, s, o, klim,
                                                                              o.viscous != TY_VISC_NONE);
      });
    else
      pr->launch(K_CELL_FAST, st, [&] {
        k_cell_fast<8, 64><<<(unsigned)((m.nci + 63) / 64), 64, 0, st>>>(m, s, o, klim,
                                                                           o.viscous != TY_VISC_NONE);
      });
    if (o.viscous != TY_VISC_NONE && m.ng > 0)
      pr->launch(K_GHOST_GRAD, st, [&] { k_ghost_grad<<<nblk(m.ng), kBlock, 0, st>>>(m, s.grad); });
    pr->launch(K_FACE_FLUX_FAST, st, [&] { k_face_flux_fast<<<nblk(m.nf), kBlock, 0, st>>>(m, s, o); });
    return cudaGetLastError();
  }
  if (o.gradmeth != TY_GRAD_NONE) {
    pr->launch(K_GRAD, st, [&] { k_grad<<<nblk(m.nci), kBlock, 0, st>>>(m, s); });
    if (m.ng > 0)
      pr->launch(K_GHOST_GRAD, st, [&] { k_ghost_grad<<<nblk(m.ng), kBlock, 0, st>>>(m, s.grad); });
  }
  if (o.postlim != TY_POSTLIM_NONE) {
    pr->launch(K_FACE_STATES, st, [&] { k_face_states<<<nblk(m.nf), kBlock, 0, st>>>(m, s, o); });
    const double klim = o.postlim == TY_POSTLIM_BARTH ? 0.5 : 1.0;
    pr->launch(K_BARTH, st, [&] { k_barth<<<nblk(m.nci), kBlock, 0, st>>>(m, s, klim); });
    pr->launch(K_FACE_FLUX_LIM, st, [&] { k_face_flux_lim<<<nblk(m.nf), kBlock, 0, st>>>(m, s, o); });
  } else {
    pr->launch(K_FACE_FLUX, st, [&] { k_face_flux<<<nblk(m.nf), kBlock, 0, st>>>(m, s, o); });
  }
  return cudaGetLastError();
}

cudaError_t residual_gather(const DevMesh& m, const DevState& s, double dt, const unsigned long long* dtbits,
                            cudaStream_t st, Prof* pr) {
  pr->launch(K_GATHER, st, [&] { k_gather<<<nblk(m.nci), kBlock, 0, st>>>(m, s, dt, dtbits); });
  return cudaGetLastError();
}

cudaError_t rk_update(const DevMesh& m, const DevState& s, const SpatOpts& o, const RkStagePlan& plan, double dt,
                      const unsigned long long* dtbits, unsigned long long* dtbits_next, double cfl,
                      cudaStream_t st, Prof* pr) {
  pr->launch(K_RK_UPDATE, st, [&] {
    k_rk_update<<<nblk(m.nci), kBlock, 0, st>>>(m, s, plan, o.gamma, dt, dtbits, dtbits_next, cfl);
  });
  return cudaGetLastError();
}

cudaError_t timestep(const DevMesh& m, const DevState& s, const SpatOpts& o, const double* cons, double cfl,
                     unsigned long long* dtbits, cudaStream_t st, Prof* pr) {
  pr->launch(K_TIMESTEP, st, [&] {
    k_timestep<<<nblk(m.nci), kBlock, 0, st>>>(m, cons, o.gamma, cfl, dtbits, s.err);
  });
  return cudaGetLastError();
}

// One stage of the ghost-row bookkeeping (GhostRk): one thread per ghost cell, [5][ng] arrays
// (gres [nstage][5][ng]), the operation order of the oracle's Runge-Kutta loop over all cells.
__global__ void k_ghost_rows(DevMesh m, const double* __restrict__ flux, GhostRk r, double gamma,
                             double* __restrict__ gcons, double* __restrict__ gres, double* __restrict__ gprim) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= m.ng) return;
  const size_t ng = m.ng;
  const int f = m.gface[g];
  double U[5], Q[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) U[v] = gcons[v * ng + g];
  for (int s = 0; s < r.stage; ++s)
#pragma unroll
    for (int v = 0; v < 5; ++v) U[v] = U[v] + r.cs[s] * gres[(s * 5 + v) * ng + g];
  cons_to_prim(gamma, U, Q);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    gprim[v * ng + g] = Q[v];
    gres[(r.stage * 5 + v) * ng + g] = flux[v * (size_t)m.ldf + f];
  }
  if (r.stage == r.nstage - 1) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double a = r.cf[0] * gres[v * ng + g];
      for (int s = 1; s < r.nstage; ++s) a = a + r.cf[s] * gres[(s * 5 + v) * ng + g];
      gcons[v * ng + g] = gcons[v * ng + g] + a;
    }
  }
}

cudaError_t ghost_rows(const DevMesh& m, const DevState& s, const SpatOpts& o, const GhostRk& r, double* gcons,
                       double* gres, double* gprim, cudaStream_t st) {
  if (m.ng > 0) k_ghost_rows<<<nblk(m.ng), kBlock, 0, st>>>(m, s.flux, r, o.gamma, gcons, gres, gprim);
  return cudaGetLastError();
}

// Typhon layout (rho[n], rhoE[n], rhou as (x,y,z)[n]) <-> SoA u0, on the device
__global__ void k_unpack_state(DevMesh m, const double* __restrict__ stage, double* __restrict__ u0) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t n = m.nci, ld = m.ldc;
  u0[c] = stage[c];
  u0[ld + c] = stage[n + c];
#pragma unroll
  for (int k = 0; k < 3; ++k) u0[(2 + k) * ld + c] = stage[2 * n + 3 * (size_t)c + k];
}
__global__ void k_pack_state(DevMesh m, const double* __restrict__ u0, double* __restrict__ stage) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t n = m.nci, ld = m.ldc;
  stage[c] = u0[c];
  stage[n + c] = u0[ld + c];
#pragma unroll
  for (int k = 0; k < 3; ++k) stage[2 * n + 3 * (size_t)c + k] = u0[(2 + k) * ld + c];
}
cudaError_t unpack_state(const DevMesh& m, const DevState& s, cudaStream_t st) {
  k_unpack_state<<<nblk(m.nci), kBlock, 0, st>>>(m, s.stage, s.u0);
  return cudaGetLastError();
}
cudaError_t pack_state(const DevMesh& m, const DevState& s, cudaStream_t st) {
  k_pack_state<<<nblk(m.nci), kBlock, 0, st>>>(m, s.u0, s.stage);
  return cudaGetLastError();
}

}  // namespace TY_KNS
}  // namespace tyk
