// Kernels of the implicit step, instantiated once per arithmetic mode after kernels.cuh.
//
// Assembly follows Typhon's order of operations so that the exact mode reproduces the CPU
// restatement bit for bit:
//   flux Jacobians       calc_jacflux.f90:49-77, calc_jac_hll.f90:46-57 (HLLC, Roe),
//                        calc_jac_rusanov.f90 (Rusanov), viscous diagonal
//                        calc_flux_viscous_cell.f90:149-158, symmetry ns_bocojacobian.f90:47-85
//                        (and, new, the far-field and no-slip wall ghost dependences folded in
//                        the same way),
//                        surface scaling flux_to_res.f90:74-80
//   BDLU blocks          build_implicit_bdlu.f90:44-83 (diagonal contributions of a cell
//                        summed in ascending face order, as the face loop there does)
//   mat-vec              SPMAT_BDLU.f90:139-157 (y = A x), :240-262 (y = z - A x)
// Reductions (dot products, norms) use a fixed two-level tree: deterministic from run to run,
// but not Typhon's sequential sum, so the Krylov iterates agree with the CPU restatement to
// rounding, not bitwise.
#pragma once
#include <algorithm>
#include <type_traits>

#include "implicit.hpp"

namespace tyk {
namespace TY_KNS {

// Jacobian of the physical flux along n, row-major (calc_jacflux.f90:49-77); q = (rho, p, u)
__device__ void jacflux(double g, const double* q, double nx, double ny, double nz, double vn, double* J) {
  const double g1 = g - 1.0, ig1 = 1.0 / g1;
  const double u[3] = {q[2], q[3], q[4]}, t[3] = {nx, ny, nz};
  const double v2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double en = ig1 * q[1] / q[0] + .5 * v2;
  J[0] = 0.0; J[1] = 0.0; J[2] = t[0]; J[3] = t[1]; J[4] = t[2];
  J[5] = vn * (g1 * v2 - g * en);
  J[6] = vn * g;
  const double c23 = g * en - .5 * g1 * v2;
#pragma unroll
  for (int k = 0; k < 3; ++k) J[7 + k] = c23 * t[k] - g1 * vn * u[k];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    J[(2 + k) * 5] = .5 * g1 * v2 * t[k] - vn * u[k];
    J[(2 + k) * 5 + 1] = g1 * t[k];
  }
  const double gn[3] = {g1 * t[0], g1 * t[1], g1 * t[2]};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) J[(2 + i) * 5 + 2 + j] = u[i] * t[j] - gn[i] * u[j];
  J[12] = J[12] + vn;
  J[18] = J[18] + vn;
  J[24] = J[24] + vn;
}

// Left and right flux Jacobians of one face, per unit surface
__device__ void face_jacobians(const SpatOpts& o, const double* L, const double* R, double nx, double ny, double nz,
                               double* JL, double* JR) {
  const double g = o.gamma;
  const double vnl = L[2] * nx + L[3] * ny + L[4] * nz;
  const double vnr = R[2] * nx + R[3] * ny + R[4] * nz;
  const double al = sqrt(g * L[1] / L[0]), ar = sqrt(g * R[1] / R[0]);
  jacflux(g, L, nx, ny, nz, vnl, JL);
  jacflux(g, R, nx, ny, nz, vnr, JR);
  if (o.scheme == TY_SCH_RUSANOV) {  // calc_jac_rusanov.f90: (A_L + ray I)/2, (A_R - ray I)/2
    const double ray = fmax(fabs(vnl) + al, fabs(vnr) + ar);
#pragma unroll
    for (int i = 0; i < 5; ++i) { JL[i * 6] = JL[i * 6] + ray; JR[i * 6] = JR[i * 6] - ray; }
#pragma unroll
    for (int k = 0; k < 25; ++k) { JL[k] = .5 * JL[k]; JR[k] = .5 * JR[k]; }
    return;
  }
  double sl, sr;
  if (o.hll_family != 0) {  // the HLLC / HLLE family's wave speeds (calc_flux_hllc.f90:86-124, calc_flux_hlle.f90:83-120)
    const double gig1 = g / (g - 1.0);
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
    double vm = rux * nx + ruy * ny + ruz * nz;
    double am = sqrt(g * roe_p / roe_rho);
    hll_speeds(o, vnl, vnr, al, ar, vm, am, sl, sr);
    if (o.hll_family == 1) {  // calc_flux_hllc.f90 passes min(sl, 0), max(sr, 0) to calc_jac_hll
      sl = fmin(sl, 0.0);
      sr = fmax(sr, 0.0);
    }
  } else {  // Roe flux: HLL Jacobian with Einfeldt's speeds from the Roe average (new)
    double t1 = sqrt(R[0] / L[0]);
    double kl = 1.0 / (1.0 + t1), kr = t1 * kl;
    double ux = kl * L[2] + kr * R[2], uy = kl * L[3] + kr * R[3], uz = kl * L[4] + kr * R[4];
    double hl = g / (g - 1.0) * L[1] / L[0] + 0.5 * (L[2] * L[2] + L[3] * L[3] + L[4] * L[4]);
    double hr = g / (g - 1.0) * R[1] / R[0] + 0.5 * (R[2] * R[2] + R[3] * R[3] + R[4] * R[4]);
    double am = sqrt((g - 1.0) * (kl * hl + kr * hr - 0.5 * (ux * ux + uy * uy + uz * uz)));
    double vm = ux * nx + uy * ny + uz * nz;
    sl = fmin(fmin(vnl - al, vm - am), 0.0);
    sr = fmax(fmax(vnr + ar, vm + am), 0.0);
  }
#pragma unroll
  for (int i = 0; i < 5; ++i) { JL[i * 6] = JL[i * 6] - sl; JR[i * 6] = JR[i * 6] - sr; }
  const double cl = sr / (sr - sl), cr = -sl / (sr - sl);
#pragma unroll
  for (int k = 0; k < 25; ++k) { JL[k] = cl * JL[k]; JR[k] = cr * JR[k]; }
}

// d(ghost conservative state)/d(inside conservative state) of a far-field face (new), rows
// and columns (rho, rhoE, rhou, rhov, rhow); false when the ghost does not depend on the inside
__device__ bool farfield_jacobian(const SpatOpts& o, double nx, double ny, double nz, const double* q, double* M) {
  const double* qi = o.farfield;
  const double vn = qi[2] * nx + qi[3] * ny + qi[4] * nz;
  const double c = sqrt(o.gamma * qi[1] / qi[0]);
#pragma unroll
  for (int k = 0; k < 25; ++k) M[k] = 0.0;
  if (vn <= -c) return false;
  const double u2 = q[2] * q[2] + q[3] * q[3] + q[4] * q[4];
  if (vn < -1e-8 * c) {
    M[5] = 0.5 * u2; M[6] = 1.0; M[7] = -q[2]; M[8] = -q[3]; M[9] = -q[4];
  } else if (vn < c) {
    M[0] = 1.0;
    M[5] = -0.5 * u2; M[7] = q[2]; M[8] = q[3]; M[9] = q[4];
    M[12] = 1.0; M[18] = 1.0; M[24] = 1.0;
  } else {
#pragma unroll
    for (int i = 0; i < 5; ++i) M[i * 6] = 1.0;
  }
  return true;
}

// face states exactly as the flux kernels of the residual build them
__device__ void implicit_face_states(const DevMesh& m, const DevState& s, const SpatOpts& o, int src, int f,
                                     double* QL, double* QR) {
  const size_t ld = m.ldc, lf = m.ldf;
  auto side_state = [&](int face, int side, double* Q) {
    if (src == 0) {
      recon(m, s, o, face, side, Q);
    } else if (src == 1) {
      const int c = side ? m.fc2[face] : m.fc1[face];
      const double* qf = side ? s.cr : s.cl;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double qc = s.prim[v * ld + c];
        double rr = s.ratio[(v < 2 ? v : 2) * ld + c];
        Q[v] = qc + rr * (qf[v * lf + face] - qc);
      }
    } else {
      const double* qf = side ? s.cr : s.cl;
#pragma unroll
      for (int v = 0; v < 5; ++v) Q[v] = qf[v * lf + face];
    }
  };
  side_state(f, 0, QL);
  const int kind = f < m.nfi ? TY_BC_INTERIOR : m.fbc[f];
  if (kind == TY_BC_PERIODIC) {
    side_state(m.part[f], 0, QR);
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
    side_state(f, 1, QR);
  }
}

// J dt / V of build_implicit_bdlu.f90:51-55: two roundings per entry in exact mode, a product
// with the per-cell quotient q = dt / V in fast mode
#if TY_FAST
#define TY_DTV(J, dt, V, q) ((J) * (q))
#else
#define TY_DTV(J, dt, V, q) ((J) * (dt) / (V))
#endif

__device__ __forceinline__ double imp_dt(const ImpState& im, const ImpArgs& a, int c) {
  return a.local_dt ? im.dtloc[c] : __longlong_as_double((long long)*a.dtg);
}

// per-cell stability time step of the implicit step (calc_ns_timestep.f90:52-103), its global
// minimum through the bit patterns, and the error word for a negative or NaN energy
__global__ void __launch_bounds__(kBlock) k_imp_dtloc(DevMesh m, const double* __restrict__ cons, double gamma,
                                                       double cfl, double* __restrict__ dtloc,
                                                       unsigned long long* dtbits, int* err) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  double dt = __longlong_as_double(0x7fefffffffffffffll);
  if (c < m.nci) {
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = cons[v * (size_t)m.ldc + c];
    double d;
    if (cell_dt(m, gamma, cfl, c, u, d)) {
      dt = d;
      dtloc[c] = d;
      if (!(d > 0.0)) flag_error(err, TY_ERR_NANDT, c);
    } else {
      dtloc[c] = 0.0;
      flag_error(err, TY_ERR_NEGENERGY, c);
    }
  }
  block_min_dt(dt, dtbits);
}

__device__ __forceinline__ void store_block(double* dst, const double* J) {
  double2* d2 = reinterpret_cast<double2*>(dst);
#pragma unroll
  for (int k = 0; k < 12; ++k) d2[k] = make_double2(J[2 * k], J[2 * k + 1]);
  dst[24] = J[24];
}
__device__ __forceinline__ void load_block(const double* src, double* J) {
  const double2* s2 = reinterpret_cast<const double2*>(src);
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    double2 t = __ldg(s2 + k);
    J[2 * k] = t.x;
    J[2 * k + 1] = t.y;
  }
  J[24] = __ldg(src + 24);
}
__device__ __forceinline__ void store_block32(float* dst, const double* J) {
  float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
  for (int k = 0; k < 6; ++k)
    d4[k] = make_float4((float)J[4 * k], (float)J[4 * k + 1], (float)J[4 * k + 2], (float)J[4 * k + 3]);
  d4[6] = make_float4((float)J[24], 0.f, 0.f, 0.f);
}
__device__ __forceinline__ void store_block32f(float* dst, const float* J) {
  float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
  for (int k = 0; k < 6; ++k) d4[k] = make_float4(J[4 * k], J[4 * k + 1], J[4 * k + 2], J[4 * k + 3]);
  d4[6] = make_float4(J[24], 0.f, 0.f, 0.f);
}
__device__ __forceinline__ void load_block32(const float* src, float* J) {
  const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    float4 t = __ldg(s4 + k);
    J[4 * k] = t.x;
    if (4 * k + 1 < 25) J[4 * k + 1] = t.y;
    if (4 * k + 2 < 25) J[4 * k + 2] = t.z;
    if (4 * k + 3 < 25) J[4 * k + 3] = t.w;
  }
}

// Face Jacobians: inviscid, + viscous diagonal, symmetry mirror, times S; then the
// off-diagonal blocks of interior faces (build_implicit_bdlu.f90:54-58)
__global__ void __launch_bounds__(128) k_imp_face(DevMesh m, DevState s, SpatOpts o, ImpState im, ImpArgs a) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  double QL[5], QR[5];
  implicit_face_states(m, s, o, a.src, f, QL, QR);
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  double JL[25], JR[25];
  face_jacobians(o, QL, QR, nx, ny, nz, JL, JR);
  if (o.viscous != TY_VISC_NONE) {
    const size_t ld = m.ldc, lf = m.ldf;
    const int icl = m.fc1[f], icr = m.fc2[f];
    const double r = o.rgas;
    const double dHL = m.vgeo[f], dHR = m.vgeo[lf + f];
    const double wx = m.vgeo[2 * lf + f], wy = m.vgeo[3 * lf + f], wz = m.vgeo[4 * lf + f];
    const double rL = s.prim[icl], rR = s.prim[icr], pL = s.prim[ld + icl], pR = s.prim[ld + icr];
    const double TL = pL / (rL * r), TR = pR / (rR * r);
    const double TH = dHR * TL + dHL * TR;
    const double rhoH = dHR * rL + dHL * rR;
    const double mu = viscosity(o, rhoH, TH);
    const double id = mu / (dHR * rL + dHL * rR) / sqrt(wx * wx + wy * wy + wz * wz);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      JR[i * 6] = JR[i * 6] - id;
      JL[i * 6] = JL[i * 6] + id;
    }
  }
  const int bkind = f >= m.nfi ? m.fbc[f] : TY_BC_INTERIOR;
  bool fold = false;
  double M[25];
  if (bkind == TY_BC_SYMMETRY) {
    const double nn[3] = {nx, ny, nz};
#pragma unroll
    for (int k = 0; k < 25; ++k) M[k] = 0.0;
#pragma unroll
    for (int i = 0; i < 5; ++i) M[i * 6] = 1.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) M[(2 + i) * 5 + 2 + j] = M[(2 + i) * 5 + 2 + j] - 2.0 * (nn[i] * nn[j]);
    fold = true;
  } else if (bkind == TY_BC_FARFIELD) {
    fold = farfield_jacobian(o, nx, ny, nz, QL, M);
  } else if (bkind == TY_BC_OUTLET_SUP) {  // ns_bocojacobian.f90: dQr/dQl = I
#pragma unroll
    for (int k = 0; k < 25; ++k) M[k] = 0.0;
#pragma unroll
    for (int i = 0; i < 5; ++i) M[i * 6] = 1.0;
    fold = true;
  } else if (bkind == TY_BC_NOSLIP) {  // new: d(2 rho u_w - m, rho E + 2 rho |u_w|^2 - 2 u_w.m)/dU
    const double w[3] = {d3(m.fwall, m.ldf, f, 0), d3(m.fwall, m.ldf, f, 1), d3(m.fwall, m.ldf, f, 2)};
#pragma unroll
    for (int k = 0; k < 25; ++k) M[k] = 0.0;
    M[0] = 1.0;
    M[5] = 2.0 * (w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    M[6] = 1.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) M[7 + j] = -2.0 * w[j];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      M[(2 + i) * 5] = 2.0 * w[i];
      M[(2 + i) * 5 + 2 + i] = -1.0;
    }
    fold = true;
  }
  if (fold) {
#pragma unroll
    for (int i = 0; i < 5; ++i)
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        double t = 0.0;
#pragma unroll
        for (int k = 0; k < 5; ++k) t = t + JR[i * 5 + k] * M[k * 5 + j];
        JL[i * 5 + j] = JL[i * 5 + j] + t;
      }
#pragma unroll
    for (int k = 0; k < 25; ++k) JR[k] = 0.0;
  }
  const double S = m.fs[f];
#pragma unroll
  for (int k = 0; k < 25; ++k) { JL[k] = S * JL[k]; JR[k] = S * JR[k]; }
  store_block(im.jacL + (size_t)f * kBlk, JL);
  store_block(im.jacR + (size_t)f * kBlk, JR);
  if (f < m.nfi) {
    const int c1 = m.fc1[f], c2 = m.fc2[f];
    const double dt1 = imp_dt(im, a, c1), dt2 = imp_dt(im, a, c2);
    const double V1 = m.cvol[c1], V2 = m.cvol[c2];
    double U[25];
#if TY_FAST
    const double q1 = dt1 / V1, q2 = dt2 / V2;
#endif
#pragma unroll
    for (int k = 0; k < 25; ++k) U[k] = +TY_DTV(JR[k], dt1, V1, q1);
    if (a.want64) store_block(im.upper + (size_t)f * kBlk, U);
    if (a.want32) store_block32(im.upper32 + (size_t)f * kBlk32, U);
#pragma unroll
    for (int k = 0; k < 25; ++k) U[k] = -TY_DTV(JL[k], dt2, V2, q2);
    if (a.want64) store_block(im.lower + (size_t)f * kBlk, U);
    if (a.want32) store_block32(im.lower32 + (size_t)f * kBlk32, U);
  }
}

// 5x5 inverse by Gauss-Jordan elimination with partial pivoting; false if singular
template <class T>
__device__ bool inv5(const T* A, T* X) {
  T a[25];
#pragma unroll
  for (int k = 0; k < 25; ++k) { a[k] = A[k]; X[k] = T(0); }
#pragma unroll
  for (int i = 0; i < 5; ++i) X[i * 6] = T(1);
#pragma unroll
  for (int col = 0; col < 5; ++col) {
    int p = col;
    T best = fabs(a[col * 5 + col]);
#pragma unroll
    for (int r = col + 1; r < 5; ++r) {
      T v = fabs(a[r * 5 + col]);
      if (v > best) { best = v; p = r; }
    }
    if (!(best > T(0))) return false;
    // row swap with compile-time indices only (selects), so that a and X stay in registers
#pragma unroll
    for (int r = col + 1; r < 5; ++r) {
      const bool sw = r == p;
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const T ta = a[col * 5 + k], tx = X[col * 5 + k];
        a[col * 5 + k] = sw ? a[r * 5 + k] : ta;
        a[r * 5 + k] = sw ? ta : a[r * 5 + k];
        X[col * 5 + k] = sw ? X[r * 5 + k] : tx;
        X[r * 5 + k] = sw ? tx : X[r * 5 + k];
      }
    }
    const T ip = T(1) / a[col * 5 + col];
#pragma unroll
    for (int k = 0; k < 5; ++k) { a[col * 5 + k] *= ip; X[col * 5 + k] *= ip; }
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      if (r == col) continue;
      const T fct = a[r * 5 + col];
#pragma unroll
      for (int k = 0; k < 5; ++k) { a[r * 5 + k] -= fct * a[col * 5 + k]; X[r * 5 + k] -= fct * X[col * 5 + k]; }
    }
  }
  return true;
}

// Diagonal block of each interior cell: identity, then the cell's faces in ascending order
// (build_implicit_bdlu.f90:52-58, 71-73); optional block-Jacobi inverse
__global__ void __launch_bounds__(128) k_imp_diag(DevMesh m, ImpState im, ImpArgs a, int want_inv, int* err) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  double D[25];
#pragma unroll
  for (int k = 0; k < 25; ++k) D[k] = 0.0;
#pragma unroll
  for (int i = 0; i < 5; ++i) D[i * 6] = 1.0;
  const double dt = imp_dt(im, a, c), V = m.cvol[c];
#if TY_FAST
  const double q = dt / V;  // one division per cell; exact mode keeps Typhon's (J dt) / V per entry
#endif
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = im.cfo[sl * (size_t)m.nci + c];
    if (e < 0) break;
    const int f = e >> 1;
    double J[25];
    if (e & 1) {
      load_block(im.jacR + (size_t)f * kBlk, J);
#pragma unroll
      for (int k = 0; k < 25; ++k) D[k] = D[k] - TY_DTV(J[k], dt, V, q);
    } else {
      load_block(im.jacL + (size_t)f * kBlk, J);
#pragma unroll
      for (int k = 0; k < 25; ++k) D[k] = D[k] + TY_DTV(J[k], dt, V, q);
    }
  }
  if (a.want64) store_block(im.diag + (size_t)c * kBlk, D);
  if (a.want32) store_block32(im.diag32 + (size_t)c * kBlk32, D);
  if (want_inv && !a.want64) {  // mixed solve: only the FP32 inverse is used, so invert in FP32
    float Df[25], Xf[25];
#pragma unroll
    for (int k = 0; k < 25; ++k) Df[k] = (float)D[k];
    if (!inv5(Df, Xf)) {
      flag_error(err, TY_ERR_STATE, c);
#pragma unroll
      for (int k = 0; k < 25; ++k) Xf[k] = 0.f;
#pragma unroll
      for (int i = 0; i < 5; ++i) Xf[i * 6] = 1.f;
    }
    store_block32f(im.dinv32 + (size_t)c * kBlk32, Xf);
  } else if (want_inv) {
    double X[25];
    if (!inv5(D, X)) {
      flag_error(err, TY_ERR_STATE, c);
#pragma unroll
      for (int k = 0; k < 25; ++k) X[k] = 0.0;
#pragma unroll
      for (int i = 0; i < 5; ++i) X[i * 6] = 1.0;
    }
    if (a.want64) store_block(im.dinv + (size_t)c * kBlk, X);
    if (a.want32) store_block32(im.dinv32 + (size_t)c * kBlk32, X);
  }
}

// right-hand side: the residual with per-cell dt (flux_to_res.f90:90-144), packed per cell
__global__ void __launch_bounds__(kBlock) k_imp_rhs(DevMesh m, DevState s, ImpState im, ImpArgs a,
                                                     double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  double R[5];
  gather_residual(m, s, c, R);
  const double coef = imp_dt(im, a, c) / m.cvol[c];
#pragma unroll
  for (int v = 0; v < 5; ++v) out[5 * (size_t)c + v] = coef * R[v];
}

__device__ __forceinline__ void mv5(const double* A, const double* x, double* t) {
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 5; ++j) s = s + A[i * 5 + j] * x[j];
    t[i] = s;
  }
}

// y = A x (z == null) or y = z - A x: diagonal block first, then the cell's interior faces in
// ascending order.  Boundary faces multiply the (zero) ghost unknowns and are skipped.
__global__ void __launch_bounds__(128) k_imp_matvec(DevMesh m, ImpState im, const double* __restrict__ x,
                                                     const double* __restrict__ z, double* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  double A[25], xv[5], t[5], yv[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) xv[v] = x[5 * (size_t)c + v];
  load_block(im.diag + (size_t)c * kBlk, A);
  mv5(A, xv, t);
  if (z) {
#pragma unroll
    for (int v = 0; v < 5; ++v) yv[v] = z[5 * (size_t)c + v] - t[v];
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) yv[v] = t[v];
  }
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = im.cfo[sl * (size_t)m.nci + c];
    if (e < 0) break;
    const int f = e >> 1;
    if (f >= m.nfi) break;
    const int nb = im.cfon[sl * (size_t)m.nci + c];
    load_block(((e & 1) ? im.lower : im.upper) + (size_t)f * kBlk, A);
#pragma unroll
    for (int v = 0; v < 5; ++v) xv[v] = x[5 * (size_t)nb + v];
    mv5(A, xv, t);
    if (z) {
#pragma unroll
      for (int v = 0; v < 5; ++v) yv[v] = yv[v] - t[v];
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) yv[v] = yv[v] + t[v];
    }
  }
  if (z) {
#pragma unroll
    for (int v = 0; v < 5; ++v) y[5 * (size_t)c + v] = yv[v];
  } else {  // S A x (the row scale is all ones outside the flexible GMRES)
#pragma unroll
    for (int v = 0; v < 5; ++v) y[5 * (size_t)c + v] = yv[v] * im.rs[v];
  }
}

// y = S A z with FP32 blocks and FP32 z, FP32 accumulation, FP64 result
__global__ void __launch_bounds__(128) k_imp_matvec32(DevMesh m, ImpState im, const float* __restrict__ z,
                                                       double* __restrict__ y) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  float A[28], xv[5], yv[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) xv[v] = z[5 * (size_t)c + v];
  load_block32(im.diag32 + (size_t)c * kBlk32, A);
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 5; ++j) s = fmaf(A[i * 5 + j], xv[j], s);
    yv[i] = s;
  }
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = im.cfo[sl * (size_t)m.nci + c];
    if (e < 0) break;
    const int f = e >> 1;
    if (f >= m.nfi) break;
    const int nb = im.cfon[sl * (size_t)m.nci + c];
    load_block32(((e & 1) ? im.lower32 : im.upper32) + (size_t)f * kBlk32, A);
#pragma unroll
    for (int v = 0; v < 5; ++v) xv[v] = z[5 * (size_t)nb + v];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      float s = yv[i];
#pragma unroll
      for (int j = 0; j < 5; ++j) s = fmaf(A[i * 5 + j], xv[j], s);
      yv[i] = s;
    }
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) y[5 * (size_t)c + v] = (double)yv[v] * im.rs[v];
}

// z = D^-1 S^-1 v, the block-Jacobi preconditioner of the flexible GMRES on its row-scaled
// system (S D)^-1: FP64 (v, dinv, z) or FP32 (v or v32, dinv32, z32)
__global__ void __launch_bounds__(128) k_imp_precond(DevMesh m, ImpState im, const double* __restrict__ v,
                                                      const float* __restrict__ v32, double* __restrict__ z,
                                                      float* __restrict__ z32) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  if (z) {
    double A[25], vv[5], t[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) vv[k] = v[5 * (size_t)c + k] * im.rsi[k];
    load_block(im.dinv + (size_t)c * kBlk, A);
    mv5(A, vv, t);
#pragma unroll
    for (int k = 0; k < 5; ++k) z[5 * (size_t)c + k] = t[k];
  } else {
    float A[28], vf[5];
    load_block32(im.dinv32 + (size_t)c * kBlk32, A);
#pragma unroll
    for (int k = 0; k < 5; ++k)
      vf[k] = v32 ? v32[5 * (size_t)c + k] * (float)im.rsi[k] : (float)(v[5 * (size_t)c + k] * im.rsi[k]);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      float s = 0.f;
#pragma unroll
      for (int j = 0; j < 5; ++j) s = fmaf(A[i * 5 + j], vf[j], s);
      z32[5 * (size_t)c + i] = s;
    }
  }
}

// initial guess of bdlu_gmres.f90:77-82: x = b / diag(i, i)
__global__ void __launch_bounds__(kBlock) k_imp_x0(DevMesh m, ImpState im, const double* __restrict__ b,
                                                    double* __restrict__ x) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
#pragma unroll
  for (int k = 0; k < 5; ++k) x[5 * (size_t)c + k] = b[5 * (size_t)c + k] / im.diag[(size_t)c * kBlk + k * 6];
}

// ---- deterministic reductions: fixed grid, block tree, then one block over the partials ----
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[kRedThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  v = threadIdx.x < kRedThreads / 32 ? sh[threadIdx.x] : 0.0;
  if (wid == 0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;  // valid in thread 0
}

inline unsigned red_grid(size_t n) {
  size_t g = (n + (size_t)kRedThreads * 4 - 1) / ((size_t)kRedThreads * 4);
  if (g < 1) g = 1;
  if (g > (size_t)kRedBlocks) g = kRedBlocks;
  return (unsigned)g;
}

// kind 0: sum a*b, kind 1: sum |a|
__global__ void __launch_bounds__(kRedThreads) k_red_part(const double* __restrict__ a, const double* __restrict__ b,
                                                           size_t n, int kind, double* __restrict__ part) {
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)kRedThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kRedThreads)
    s += kind == 0 ? a[i] * b[i] : fabs(a[i]);
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// out[k] = sum of part[k * stride + 0 .. nb-1], one block per k
__global__ void __launch_bounds__(kRedThreads) k_red_final(const double* __restrict__ part, int nb, size_t stride,
                                                            double* __restrict__ out) {
  const double* p = part + blockIdx.x * stride;
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += kRedThreads) s += p[i];
  s = block_sum(s);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// ---- BiCGSTAB of bdlu_bicgstab.f90:52-75, scalars kept on the device: sc[0] rho1, sc[1] rho0,
// sc[2] alpha, sc[3] omega (of the previous iteration), sc[4] r2.v, sc[5] t.s, sc[6] t.t,
// sc[7] err.  Each kernel derives the step's alpha, beta, omega from them itself.
// p = r1 (first iteration) or r1 + beta (p - omega v), beta = (rho1/rho0)(alpha/omega)
__global__ void k_bicg_p(const double* __restrict__ r1, const double* __restrict__ v, double* __restrict__ p,
                         const double* __restrict__ sc, int first, size_t n) {
  const double beta = first ? 0.0 : (sc[0] / sc[1]) * (sc[2] / sc[3]);
  const double om = sc[3];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (first) p[i] = r1[i];
    else {
      const double q = p[i] - om * v[i];
      p[i] = r1[i] + beta * q;
    }
  }
}
// s = r1 - alpha v, alpha = rho1 / (r2.v)
__global__ void k_bicg_s(const double* __restrict__ r1, const double* __restrict__ v, double* __restrict__ s,
                         const double* __restrict__ sc, size_t n) {
  const double alpha = sc[0] / sc[4];
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s[i] = r1[i] - alpha * v[i];
}
// partial sums of t.s and t.t
__global__ void __launch_bounds__(kRedThreads) k_bicg_ts(const double* __restrict__ t, const double* __restrict__ s,
                                                          size_t n, double* __restrict__ part) {
  double a = 0.0, b = 0.0;
  for (size_t i = blockIdx.x * (size_t)kRedThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kRedThreads) {
    a += t[i] * s[i];
    b += t[i] * t[i];
  }
  a = block_sum(a);
  b = block_sum(b);
  if (threadIdx.x == 0) { part[blockIdx.x] = a; part[kRedBlocks + blockIdx.x] = b; }
}
// omega = (t.s)/(t.t); err partials of |alpha p + omega s|; x += alpha p + omega s; r1 = s - omega t
__global__ void __launch_bounds__(kRedThreads) k_bicg_update(double* __restrict__ x, double* __restrict__ r1,
                                                              const double* __restrict__ p,
                                                              const double* __restrict__ s,
                                                              const double* __restrict__ t,
                                                              const double* __restrict__ sc, size_t n,
                                                              double* __restrict__ part) {
  const double alpha = sc[0] / sc[4], omega = sc[5] / sc[6];
  double e = 0.0;
  for (size_t i = blockIdx.x * (size_t)kRedThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kRedThreads) {
    const double ap = alpha * p[i], os = omega * s[i];
    e += fabs(ap + os);
    x[i] = x[i] + ap + os;
    r1[i] = s[i] - omega * t[i];
  }
  e = block_sum(e);
  if (threadIdx.x == 0) part[blockIdx.x] = e;
}
// end of an iteration: rho0 = rho1, alpha and omega kept for the next beta
__global__ void k_bicg_shift(double* sc) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double alpha = sc[0] / sc[4], omega = sc[5] / sc[6];
    sc[1] = sc[0];
    sc[2] = alpha;
    sc[3] = omega;
  }
}

// modified Gram-Schmidt pass: w = w - hprev * vprev (when vprev), then partial sums of w . vnext
__global__ void __launch_bounds__(kRedThreads) k_mgs_pass(const double* __restrict__ vprev,
                                                           const double* __restrict__ hprev, double* __restrict__ w,
                                                           const double* __restrict__ vnext, size_t n,
                                                           double* __restrict__ part) {
  const double h = vprev ? *hprev : 0.0;
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)kRedThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kRedThreads) {
    double wi = w[i];
    if (vprev) {
      wi = wi - h * vprev[i];
      w[i] = wi;
    }
    s += wi * (vnext ? vnext[i] : wi);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Krylov basis pass of the flexible GMRES (basis vector i at V + i ldv, stored as T):
//   extend 0: out_i = V_i . src (i < nv), out_nv = src . src
//   extend 1: v = (src - sum_{i<nv} c_i V_i) s is stored as V_nv (rounded to T), then
//             out_i = V_i . v (i < nv), out_nv = v . v, of the stored values
// An FP64 basis is swept in FP64; an FP32 basis (mixed-precision solve) in FP32 arithmetic
// with FP64 block sums.  The first form projects A z_j on the basis; the second forms the next
// basis vector and the new column of the basis' Gram matrix in the same sweep, so one iteration reads the basis
// twice and synchronises with the host once.  One row per thread per trip: the row's basis
// entries are loaded together and kept in registers; the per-thread sums live in shared
// memory.  Each block reduces its sums once, writes one partial per output, and the last block
// to finish adds the partials in block order: one launch, the same result for the same grid.
template <int J, class T>
__global__ void __launch_bounds__(kCgsThreads) k_basis_pass(T* V, size_t ldv, int nv, const double* __restrict__ c,
                                                             const double* __restrict__ src,
                                                             const double* __restrict__ sp, int extend, size_t n,
                                                             double* __restrict__ part, unsigned* __restrict__ done,
                                                             double* __restrict__ out) {
  __shared__ double cl[J];
  __shared__ double acc[J + 1][kCgsThreads];
  __shared__ bool last;
  const int t = threadIdx.x;
  if (t < J) cl[t] = (extend && t < nv) ? c[t] : 0.0;
#pragma unroll
  for (int i = 0; i <= J; ++i) acc[i][t] = 0.0;
  const double sc = extend ? *sp : 1.0;
  __syncthreads();
  T* vout = V + (size_t)nv * ldv;
  if constexpr (std::is_same<T, double>::value && J <= 16) {
    // short bases: per-thread sums in registers, written to shared memory once
    double ad[J];
#pragma unroll
    for (int i = 0; i < J; ++i) ad[i] = 0.0;
    double xx = 0.0;
    for (size_t k = blockIdx.x * (size_t)kCgsThreads + t; k < n; k += (size_t)gridDim.x * kCgsThreads) {
      double v[J];
      const double* pv = V + k;
#pragma unroll
      for (int i = 0; i < J; ++i) {
        v[i] = i < nv ? *pv : 0.0;
        pv += ldv;
      }
      double x = src[k];
      if (extend) {
#pragma unroll
        for (int i = 0; i < J; ++i)
          if (i < nv) x = x - cl[i] * v[i];
        x = x * sc;
        vout[k] = x;
      }
#pragma unroll
      for (int i = 0; i < J; ++i)
        if (i < nv) ad[i] += v[i] * x;
      xx += x * x;
    }
#pragma unroll
    for (int i = 0; i < J; ++i)
      if (i < nv) acc[i][t] = ad[i];
    acc[nv][t] = xx;
  } else if constexpr (std::is_same<T, double>::value) {
    double xx = 0.0;
    for (size_t k = blockIdx.x * (size_t)kCgsThreads + t; k < n; k += (size_t)gridDim.x * kCgsThreads) {
      double v[J];
      const double* pv = V + k;
#pragma unroll
      for (int i = 0; i < J; ++i) {
        v[i] = i < nv ? *pv : 0.0;
        pv += ldv;
      }
      double x = src[k];
      if (extend) {
#pragma unroll
        for (int i = 0; i < J; ++i)
          if (i < nv) x = x - cl[i] * v[i];
        x = x * sc;
        vout[k] = x;
      }
#pragma unroll
      for (int i = 0; i < J; ++i)
        if (i < nv) acc[i][t] += v[i] * x;
      xx += x * x;
    }
    acc[nv][t] = xx;
  } else {
    // FP32 basis: FP32 arithmetic per row (GB300 issues FP32 at about 60x its FP64 rate),
    // per-thread sums in FP32 registers over the thread's rows, FP64 from the block sums on
    float cf[J], af[J];
#pragma unroll
    for (int i = 0; i < J; ++i) {
      cf[i] = (float)cl[i];
      af[i] = 0.f;
    }
    const float sf = (float)sc;
    float xx = 0.f;
    // R rows per trip (R x nv independent 4-byte loads in flight) for the short bases
    constexpr int R = J <= 8 ? 4 : (J <= 16 ? 2 : 1);
    const size_t stride = (size_t)gridDim.x * kCgsThreads;
    for (size_t k0 = blockIdx.x * (size_t)kCgsThreads + t; k0 < n; k0 += R * stride) {
      float v[R][J], x[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const size_t k = k0 + r * stride;
        const bool ok = k < n;
        const float* pv = V + k;
#pragma unroll
        for (int i = 0; i < J; ++i) {
          v[r][i] = (ok && i < nv) ? *pv : 0.f;
          pv += ldv;
        }
        x[r] = ok ? (float)src[k] : 0.f;
      }
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (extend) {
#pragma unroll
          for (int i = 0; i < J; ++i)
            if (i < nv) x[r] = fmaf(-cf[i], v[r][i], x[r]);
          x[r] = x[r] * sf;
          if (k0 + r * stride < n) vout[k0 + r * stride] = x[r];
        }
#pragma unroll
        for (int i = 0; i < J; ++i)
          if (i < nv) af[i] = fmaf(v[r][i], x[r], af[i]);
        xx = fmaf(x[r], x[r], xx);
      }
    }
#pragma unroll
    for (int i = 0; i < J; ++i)
      if (i < nv) acc[i][t] = (double)af[i];
    acc[nv][t] = (double)xx;
  }
  __syncthreads();
  const int nout = nv + 1;
  const int lane = t & 31, wid = t >> 5;
  for (int i = wid; i < nout; i += kCgsThreads / 32) {
    double x = 0.0;
#pragma unroll
    for (int q = 0; q < kCgsThreads / 32; ++q) x += acc[i][q * 32 + lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) part[(size_t)i * kRedBlocks + blockIdx.x] = x;
  }
  __threadfence();
  __syncthreads();
  if (t == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  for (int i = wid; i < nout; i += kCgsThreads / 32) {
    const double* p = part + (size_t)i * kRedBlocks;
    double x = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) x += __ldcg(p + b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) out[i] = x;
  }
  if (t == 0) *done = 0u;  // ready for the next launch on the stream
}

__global__ void k_scale(const double* __restrict__ w, double s, double* __restrict__ v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    v[i] = s * w[i];
}

// x = x + y_j V_j over j (descending order when asked, as bdlu_gmres.f90:176-187 does)
__global__ void k_axpy_multi(double* __restrict__ x, const double* __restrict__ V, const float* __restrict__ V32,
                             size_t ldv, int j, const double* __restrict__ y, int descending, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    double xk = x[k];
    for (int q = 0; q < j; ++q) {
      const int i = descending ? j - 1 - q : q;
      const double vi = V ? V[i * ldv + k] : (double)V32[i * ldv + k];
      xk = xk + y[i] * vi;
    }
    x[k] = xk;
  }
}

// U += x (update_field.f90:38) on the resident state; partial sums of |x| per variable
__global__ void __launch_bounds__(kRedThreads) k_imp_update(DevMesh m, double* __restrict__ u0,
                                                             const double* __restrict__ x, double* __restrict__ part) {
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int c = blockIdx.x * kRedThreads + threadIdx.x; c < m.nci; c += gridDim.x * kRedThreads) {
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double d = x[5 * (size_t)c + v];
      u0[v * (size_t)m.ldc + c] = u0[v * (size_t)m.ldc + c] + d;
      s[v] += fabs(d);
    }
    const double mx = x[5 * (size_t)c + 2], my = x[5 * (size_t)c + 3], mz = x[5 * (size_t)c + 4];
    s[5] += sqrt(mx * mx + my * my + mz * mz);
  }
#pragma unroll
  for (int v = 0; v < 6; ++v) {
    double t = block_sum(s[v]);
    if (threadIdx.x == 0) part[(size_t)v * kRedBlocks + blockIdx.x] = t;
  }
}

// unscaled residual norms per variable: sum (b_c V_c / dt_c)^2
__global__ void __launch_bounds__(kRedThreads) k_imp_resnorm(DevMesh m, ImpState im, ImpArgs a,
                                                              const double* __restrict__ b, double* __restrict__ part) {
  double s[5] = {0, 0, 0, 0, 0};
  for (int c = blockIdx.x * kRedThreads + threadIdx.x; c < m.nci; c += gridDim.x * kRedThreads) {
    const double k = m.cvol[c] / imp_dt(im, a, c);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double r = b[5 * (size_t)c + v] * k;
      s[v] += r * r;
    }
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double t = block_sum(s[v]);
    if (threadIdx.x == 0) part[(size_t)v * kRedBlocks + blockIdx.x] = t;
  }
}

// Jacobian-free products: the perturbed state U + eps z (SoA), then w = z - (R(U + eps z) - R(U)) / eps
__global__ void k_imp_perturb(DevMesh m, const double* __restrict__ u0, const double* __restrict__ z, double eps,
                              double* __restrict__ up) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
#pragma unroll
  for (int v = 0; v < 5; ++v) up[v * (size_t)m.ldc + c] = u0[v * (size_t)m.ldc + c] + eps * z[5 * (size_t)c + v];
}
// w = rs (z - (rp - r0) inv_eps) per packed entry (rs of its variable i mod 5); rp null: w = rs z
__global__ void k_imp_fd(const double* __restrict__ z, const float* __restrict__ z32, const double* __restrict__ rp,
                         const double* __restrict__ r0, double inv_eps, Row5 rs, double* __restrict__ w, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double zi = z ? z[i] : (double)z32[i];
    const double d = rp ? zi - (rp[i] - (r0 ? r0[i] : 0.0)) * inv_eps : zi;
    w[i] = d * rs.v[i % 5];
  }
}

// ---------------------------------------------------------------------------
// launchers
inline unsigned grid_of(size_t n, int b) { return (unsigned)((n + b - 1) / b); }

cudaError_t imp_dtloc(const DevMesh& m, const DevState& s, const SpatOpts& o, const ImpState& im, double cfl,
                      unsigned long long* dtbits, cudaStream_t st) {
  k_imp_dtloc<<<nblk(m.nci), kBlock, 0, st>>>(m, s.u0, o.gamma, cfl, im.dtloc, dtbits, s.err);
  return cudaGetLastError();
}

cudaError_t imp_assemble(const DevMesh& m, const DevState& s, const SpatOpts& o, const ImpState& im,
                         const ImpArgs& a, cudaStream_t st, Prof* pr) {
  pr->launch(K_IMP_FACE, st, [&] { k_imp_face<<<grid_of(m.nf, 128), 128, 0, st>>>(m, s, o, im, a); });
  pr->launch(K_IMP_DIAG, st, [&] { k_imp_diag<<<grid_of(m.nci, 128), 128, 0, st>>>(m, im, a, 1, s.err); });
  return cudaGetLastError();
}

cudaError_t imp_rhs(const DevMesh& m, const DevState& s, const ImpState& im, const ImpArgs& a, double* out,
                    cudaStream_t st) {
  k_imp_rhs<<<nblk(m.nci), kBlock, 0, st>>>(m, s, im, a, out);
  return cudaGetLastError();
}

cudaError_t imp_matvec(const DevMesh& m, const ImpState& im, const double* x, const double* z, double* y,
                       cudaStream_t st, Prof* pr) {
  pr->launch(K_IMP_MATVEC, st, [&] { k_imp_matvec<<<grid_of(m.nci, 128), 128, 0, st>>>(m, im, x, z, y); });
  return cudaGetLastError();
}

cudaError_t imp_matvec32(const DevMesh& m, const ImpState& im, const float* z, double* y, cudaStream_t st,
                         Prof* pr) {
  pr->launch(K_IMP_MATVEC, st, [&] { k_imp_matvec32<<<grid_of(m.nci, 128), 128, 0, st>>>(m, im, z, y); });
  return cudaGetLastError();
}

cudaError_t imp_precond(const DevMesh& m, const ImpState& im, const double* v, const float* v32, double* z,
                        float* z32, cudaStream_t st, Prof* pr) {
  pr->launch(K_IMP_PRECOND, st,
             [&] { k_imp_precond<<<grid_of(m.nci, 128), 128, 0, st>>>(m, im, v, v32, z, z32); });
  return cudaGetLastError();
}

cudaError_t imp_x0_diag(const DevMesh& m, const ImpState& im, const double* b, double* x, cudaStream_t st) {
  k_imp_x0<<<nblk(m.nci), kBlock, 0, st>>>(m, im, b, x);
  return cudaGetLastError();
}

cudaError_t imp_dot(const double* a, const double* b, size_t n, double* part, double* out, cudaStream_t st) {
  const unsigned g = red_grid(n);
  k_red_part<<<g, kRedThreads, 0, st>>>(a, b, n, 0, part);
  k_red_final<<<1, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, out);
  return cudaGetLastError();
}

// update_field.f90:45-60's residual terms of an explicit step: per block the sums over its
// interior cells of |acc_rho|, |acc_rhoE| and |acc_m| (acc: the step's combination of stage
// residuals, [5][ld])
__global__ void __launch_bounds__(kRedThreads) k_res_l1(int nci, const double* __restrict__ acc, size_t ld,
                                                         double* __restrict__ part) {
  double a = 0.0, b = 0.0, q = 0.0;
  for (int c = blockIdx.x * kRedThreads + threadIdx.x; c < nci; c += gridDim.x * kRedThreads) {
    a += fabs(acc[c]);
    b += fabs(acc[ld + c]);
    const double mx = acc[2 * ld + c], my = acc[3 * ld + c], mz = acc[4 * ld + c];
    q += sqrt(mx * mx + my * my + mz * mz);
  }
  a = block_sum(a);
  b = block_sum(b);
  q = block_sum(q);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = a;
    part[kRedBlocks + blockIdx.x] = b;
    part[2 * kRedBlocks + blockIdx.x] = q;
  }
}

cudaError_t res_l1(int nci, const double* acc, size_t ld, double* part, double* out, cudaStream_t st) {
  const unsigned g = red_grid((size_t)nci);
  k_res_l1<<<g, kRedThreads, 0, st>>>(nci, acc, ld, part);
  k_red_final<<<3, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, out);
  return cudaGetLastError();
}

cudaError_t imp_asum(const double* a, size_t n, double* part, double* out, cudaStream_t st) {
  const unsigned g = red_grid(n);
  k_red_part<<<g, kRedThreads, 0, st>>>(a, nullptr, n, 1, part);
  k_red_final<<<1, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, out);
  return cudaGetLastError();
}

cudaError_t imp_mgs_pass(const double* vprev, const double* hprev, double* w, const double* vnext, size_t n,
                         double* part, double* out, cudaStream_t st) {
  const unsigned g = red_grid(n);
  k_mgs_pass<<<g, kRedThreads, 0, st>>>(vprev, hprev, w, vnext, n, part);
  k_red_final<<<1, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, out);
  return cudaGetLastError();
}

// blocks of a basis pass: the resident blocks of the whole GPU (at most kRedBlocks), fewer
// for short vectors; a fixed function of n and the device, so sums repeat from run to run
template <int J, class T>
unsigned basis_grid(size_t n) {
  static const unsigned cap = [] {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_basis_pass<J, T>, kCgsThreads, 0);
    const long c = (long)std::max(sms, 1) * std::max(per, 1);
    return (unsigned)std::min<long>(c, kRedBlocks);
  }();
  const size_t g = (n + kCgsThreads - 1) / kCgsThreads;
  return (unsigned)std::max<size_t>(1, std::min<size_t>(g, cap));
}

template <int J, class T>
void basis_launch_j(T* V, size_t ldv, int nv, const double* c, const double* src, const double* sp, int extend,
                    size_t n, double* part, unsigned* done, double* out, cudaStream_t st) {
  k_basis_pass<J, T><<<basis_grid<J, T>(n), kCgsThreads, 0, st>>>(V, ldv, nv, c, src, sp, extend, n, part, done, out);
}

// The unrolled loops of a sweep run J slots per entry whatever nv is, so an FP64 sweep (bound
// by the FP64 pipe) takes the smallest even J >= nv; an FP32 sweep (bound by HBM) takes 8, 16
// or 32.
template <class T>
void basis_launch(T* V, size_t ldv, int nv, const double* c, const double* src, const double* sp, int extend,
                  size_t n, double* part, unsigned* done, double* out, cudaStream_t st) {
  if constexpr (std::is_same<T, double>::value) {
    switch ((nv + 1) / 2) {
      case 0:
      case 1: basis_launch_j<2>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
      case 2: basis_launch_j<4>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
      case 3: basis_launch_j<6>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
      case 4: basis_launch_j<8>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
      case 5: basis_launch_j<10>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
      case 6: basis_launch_j<12>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
      case 7: basis_launch_j<14>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
      case 8: basis_launch_j<16>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
      default: basis_launch_j<kMaxCgs>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st); return;
    }
  } else {
    if (nv <= 8) basis_launch_j<8>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st);
    else if (nv <= 16) basis_launch_j<16>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st);
    else basis_launch_j<kMaxCgs>(V, ldv, nv, c, src, sp, extend, n, part, done, out, st);
  }
}

cudaError_t imp_basis_pass(double* V, float* V32, size_t ldv, int nv, const double* c, const double* src,
                           const double* sp, int extend, size_t n, double* part, unsigned* done, double* out,
                           cudaStream_t st, Prof* pr) {
  if (nv < 0 || nv > kMaxCgs) return cudaErrorInvalidValue;
  pr->launch(K_IMP_ORTHO, st, [&] {
    if (V32) basis_launch(V32, ldv, nv, c, src, sp, extend, n, part, done, out, st);
    else basis_launch(V, ldv, nv, c, src, sp, extend, n, part, done, out, st);
  });
  return cudaGetLastError();
}

cudaError_t imp_bicgstab_iter(const DevMesh& m, const ImpState& im, double* x, double* r1, const double* r2,
                              double* p, double* v, double* s, double* t, int first, double* part, double* sc,
                              cudaStream_t st, Prof* pr) {
  const size_t n = 5 * (size_t)m.nci;
  const unsigned gv = (unsigned)std::min<size_t>(grid_of(n, 256), 4 * kRedBlocks);
  const unsigned g = red_grid(n);
  k_red_part<<<g, kRedThreads, 0, st>>>(r1, r2, n, 0, part);                // rho1 = r1.r2
  k_red_final<<<1, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, sc + 0);
  k_bicg_p<<<gv, 256, 0, st>>>(r1, v, p, sc, first, n);
  pr->launch(K_IMP_MATVEC, st, [&] { k_imp_matvec<<<grid_of(m.nci, 128), 128, 0, st>>>(m, im, p, nullptr, v); });
  k_red_part<<<g, kRedThreads, 0, st>>>(r2, v, n, 0, part);                 // r2.v
  k_red_final<<<1, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, sc + 4);
  k_bicg_s<<<gv, 256, 0, st>>>(r1, v, s, sc, n);
  pr->launch(K_IMP_MATVEC, st, [&] { k_imp_matvec<<<grid_of(m.nci, 128), 128, 0, st>>>(m, im, s, nullptr, t); });
  k_bicg_ts<<<g, kRedThreads, 0, st>>>(t, s, n, part);
  k_red_final<<<2, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, sc + 5);
  k_bicg_update<<<g, kRedThreads, 0, st>>>(x, r1, p, s, t, sc, n, part);
  k_red_final<<<1, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, sc + 7);
  k_bicg_shift<<<1, 32, 0, st>>>(sc);
  return cudaGetLastError();
}

cudaError_t imp_scale(const double* w, double s, double* v, size_t n, cudaStream_t st) {
  k_scale<<<std::min<size_t>(grid_of(n, 256), 4 * kRedBlocks), 256, 0, st>>>(w, s, v, n);
  return cudaGetLastError();
}

cudaError_t imp_axpy_multi(double* x, const double* V, const float* V32, size_t ldv, int j, const double* y,
                           int descending, size_t n, cudaStream_t st) {
  k_axpy_multi<<<std::min<size_t>(grid_of(n, 256), 4 * kRedBlocks), 256, 0, st>>>(x, V, V32, ldv, j, y,
                                                                                 descending, n);
  return cudaGetLastError();
}

cudaError_t imp_update_state(const DevMesh& m, DevState& s, const double* x, double* part, double* out,
                             cudaStream_t st) {
  const unsigned g = red_grid(m.nci);
  k_imp_update<<<g, kRedThreads, 0, st>>>(m, s.u0, x, part);
  k_red_final<<<6, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, out);
  return cudaGetLastError();
}

cudaError_t imp_perturb(const DevMesh& m, const double* u0, const double* z, double eps, double* up,
                        cudaStream_t st) {
  k_imp_perturb<<<nblk(m.nci), kBlock, 0, st>>>(m, u0, z, eps, up);
  return cudaGetLastError();
}

cudaError_t imp_fd_combine(const double* z, const float* z32, const double* rp, const double* r0, double inv_eps,
                           Row5 rs, double* w, size_t n, cudaStream_t st) {
  k_imp_fd<<<std::min<size_t>(grid_of(n, 256), 4 * kRedBlocks), 256, 0, st>>>(z, z32, rp, r0, inv_eps, rs, w, n);
  return cudaGetLastError();
}

__global__ void k_to_f32(const double* __restrict__ x, float* __restrict__ y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}
cudaError_t imp_to_f32(const double* x, float* y, size_t n, cudaStream_t st) {
  k_to_f32<<<std::min<size_t>(grid_of(n, 256), 4 * kRedBlocks), 256, 0, st>>>(x, y, n);
  return cudaGetLastError();
}

cudaError_t imp_res_norms(const DevMesh& m, const ImpState& im, const ImpArgs& a, const double* b, double* part,
                          double* out, cudaStream_t st) {
  const unsigned g = red_grid(m.nci);
  k_imp_resnorm<<<g, kRedThreads, 0, st>>>(m, im, a, b, part);
  k_red_final<<<5, kRedThreads, 0, st>>>(part, (int)g, kRedBlocks, out);
  return cudaGetLastError();
}

}  // namespace TY_KNS
}  // namespace tyk
