// Adjoint (vector-Jacobian product) of the residual, instantiated per mode after kernels.cuh.  New: Typhon has no adjoint (its inverse mode differentiates by finite
// differences, SOURCE/MAIN/inverse_calc_sensi.f90).
//
// R_c = dt/V_c sum_f (+-) F_f(U) S_f with face states Q_L = prim(U_fc1), Q_R = prim(U_fc2) or
// the boundary state built from Q_L (periodic: the partner's inside cell).  Given lambda_R,
//   lambda_F(f) = S_f (dt/V_fc2 lambda_R(fc2) [interior faces] - dt/V_fc1 lambda_R(fc1)),
//   lambda_U   += (dF/dU_L)^T lambda_F on fc1 and (dF/dU_R)^T lambda_F on the right cell,
// the face loop reversed into a gather: a face kernel writes both products, a cell kernel
// sums a cell's faces (and, for a periodic boundary face, the product of its partner face,
// whose right state is this cell).  The products come from reverse-mode derivatives written
// by hand (adjoint_flux.cuh) of the same formulas as the exact-mode residual, traversed
// backwards: flux, boundary state, cons -> prim.  One thread per face, no dual numbers.
#pragma once
#include "adjoint.hpp"
#include "adjoint_flux.cuh"

namespace tyk {
namespace TY_KNS {

using namespace adflux;

// right state of a boundary face built from the left one (first order)
__device__ void bc_state(const DevMesh& m, const SpatOpts& o, int f, int kind, const double* QL, double* QR) {
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  if (kind == TY_BC_SYMMETRY) {
    double dn = 2.0 * (QL[2] * nx + QL[3] * ny + QL[4] * nz);
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
      for (int v = 0; v < 5; ++v) QR[v] = qi[v];
    } else if (vn < -1e-8 * c) {
      QR[0] = qi[0]; QR[1] = QL[1]; QR[2] = qi[2]; QR[3] = qi[3]; QR[4] = qi[4];
    } else if (vn < c) {
      QR[0] = QL[0]; QR[1] = qi[1]; QR[2] = QL[2]; QR[3] = QL[3]; QR[4] = QL[4];
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) QR[v] = QL[v];
    }
  }
}

// reverse of bc_state (QR built from QL): QLb += (dQR/dQL)^T QRb
__device__ void bc_state_vjp(const DevMesh& m, const SpatOpts& o, int f, int kind, const double* QRb, double* QLb) {
  const double n[3] = {d3(m.fn, m.ldf, f, 0), d3(m.fn, m.ldf, f, 1), d3(m.fn, m.ldf, f, 2)};
  if (kind == TY_BC_SYMMETRY) {
    QLb[0] += QRb[0];
    QLb[1] += QRb[1];
    const double s = QRb[2] * n[0] + QRb[3] * n[1] + QRb[4] * n[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) QLb[2 + k] += QRb[2 + k] - 2.0 * s * n[k];
  } else if (kind == TY_BC_WALL || kind == TY_BC_NOSLIP) {
    if (kind == TY_BC_NOSLIP) QLb[0] += QRb[0];
    else QLb[1] += QRb[0];
    QLb[1] += QRb[1];
#pragma unroll
    for (int k = 0; k < 3; ++k) QLb[2 + k] -= QRb[2 + k];
  } else {
    const double* qi = o.farfield;
    const double vn = qi[2] * n[0] + qi[3] * n[1] + qi[4] * n[2];
    const double c = ::sqrt(o.gamma * qi[1] / qi[0]);
    if (vn <= -c) return;
    if (vn < -1e-8 * c) { QLb[1] += QRb[1]; return; }
    if (vn < c) { QLb[0] += QRb[0]; QLb[2] += QRb[2]; QLb[3] += QRb[3]; QLb[4] += QRb[4]; return; }
#pragma unroll
    for (int v = 0; v < 5; ++v) QLb[v] += QRb[v];
  }
}


// per face: lambda_F, then (dF/dU_L)^T lambda_F and (dF/dU_R)^T lambda_F into lam_face [10][ldf]
// (zero right product on a non-periodic boundary face, whose right state is built from the
// left one)
template <int SCH>
__global__ void __launch_bounds__(128) k_adj_face(DevMesh m, SpatOpts o, const double* __restrict__ u,
                                                  const double* __restrict__ lamR, double dt,
                                                  double* __restrict__ lam_face) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const size_t ld = m.ldc, lf = m.ldf;
  const int c1 = m.fc1[f];
  const int kind = f < m.nfi ? TY_BC_INTERIOR : m.fbc[f];
  const bool two = kind == TY_BC_INTERIOR || kind == TY_BC_PERIODIC;
  const int cr = kind == TY_BC_INTERIOR ? m.fc2[f] : (kind == TY_BC_PERIODIC ? m.fc1[m.part[f]] : c1);
  const double S = m.fs[f];
  double Fb[5], uL[5], uR[5], QL[5], QR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double a = -(dt / m.cvol[c1]) * lamR[v * ld + c1];
    if (kind == TY_BC_INTERIOR) a = a + (dt / m.cvol[cr]) * lamR[v * ld + cr];
    Fb[v] = S * a;
    uL[v] = u[v * ld + c1];
    uR[v] = u[v * ld + cr];
  }
  const double irL = prim_r(o.gamma, uL, QL);
  const double irR = two ? prim_r(o.gamma, uR, QR) : 0.0;
  if (!two) bc_state(m, o, f, kind, QL, QR);
  double QLb[5] = {0, 0, 0, 0, 0}, QRb[5] = {0, 0, 0, 0, 0};
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  if constexpr (SCH == TY_SCH_HLLC) hllc_vjp(o.gamma, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  else if constexpr (SCH == TY_SCH_RUSANOV) rusanov_vjp(o.gamma, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  else roe_vjp(o.gamma, o.entropy_fix, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  if (!two) bc_state_vjp(m, o, f, kind, QRb, QLb);
  double ULb[5] = {0, 0, 0, 0, 0}, URb[5] = {0, 0, 0, 0, 0};
  prim_vjp(o.gamma, uL, irL, QLb, ULb);
  if (two) prim_vjp(o.gamma, uR, irR, QRb, URb);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    lam_face[v * lf + f] = ULb[v];
    lam_face[(5 + v) * lf + f] = URb[v];
  }
}

// ---- second order: least-squares gradients, MUSCL or MUSCL-UNS with no limiter or the van
// Albada limiter, Typhon's Barth post-limiter frozen, on meshes whose boundaries are periodic.
// The reconstruction of one face side (recon, owner cell c, cells i1 = fc1, i2 = fc2 of the
// owner face F) is
//   q = q_c + r_c (G_c . CF + sg (u . CF)),  g = G_c . u,  LR = (q_i2 - q_i1) / dLR,
//   sg = phi(2g - LR, LR) - g (MUSCL, tvdgradstr) or phi(g, LR) - g (MUSCL-UNS, tvdgraduns),
//   phi = 0: sg = LR - g,
// with phi(a, b) = a b (a + b) / (a^2 + b^2) where a b > 0, else 0 (smooth van Albada), and
// r_c the cell's Barth ratio for the variable's group (postlimit_barth.f90:42-223), held
// constant (1 without a post-limiter): the adjoint of the frozen limiter scales the
// increment's adjoint by r_c.
// reverse of one face side: Qb -> rec[0..4] adjoint of q_c, rec[5..19] of G_c (3 per
// variable), rec[20..24] of LR over dLR (+ to i2, - to i1)
__device__ void recon_vjp(const DevMesh& m, const DevState& s, const SpatOpts& o, int F, int side,
                          const double* Qb, const double* ratio, double* rec) {
  const size_t ld = m.ldc, lf = m.ldf;
  const int icl = m.fc1[F], icr = m.fc2[F];
  const int c = side ? icr : icl;
  const double ux = m.uLR[F], uy = m.uLR[lf + F], uz = m.uLR[2 * lf + F];
  const double idLR = 1.0 / m.dLR[F];
  const double* CF = side ? m.RF : m.LF;
  const double cx = CF[F], cy = CF[lf + F], cz = CF[2 * lf + F];
  const double uc = ux * cx + uy * cy + uz * cz;
  const bool uns = o.highres == TY_HRES_MUSCLUNS;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double gx = s.grad[(3 * v) * ld + c], gy = s.grad[(3 * v + 1) * ld + c], gz = s.grad[(3 * v + 2) * ld + c];
    const double LR = (s.prim[v * ld + icr] - s.prim[v * ld + icl]) * idLR;
    const double g = gx * ux + gy * uy + gz * uz;
    const double qb = Qb[v], db = ratio[v < 2 ? v : 2] * qb, sgb = db * uc;
    double gb, LRb;
    if (o.limiter == TY_LIM_NONE) {
      LRb = sgb;
      gb = -sgb;
    } else {
      const double a = uns ? g : 2.0 * g - LR, b = LR;
      double pa = 0.0, pb = 0.0;
      if (a * b > 0.0) {
        const double D = a * a + b * b, iD2 = 1.0 / (D * D);
        pa = b * b * (b * b + 2.0 * a * b - a * a) * iD2;
        pb = a * a * (a * a + 2.0 * a * b - b * b) * iD2;
      }
      if (uns) {
        gb = sgb * pa - sgb;
        LRb = sgb * pb;
      } else {
        gb = 2.0 * sgb * pa - sgb;
        LRb = sgb * pb - sgb * pa;
      }
    }
    rec[v] = qb;
    rec[5 + 3 * v] = db * cx + gb * ux;
    rec[6 + 3 * v] = db * cy + gb * uy;
    rec[7 + 3 * v] = db * cz + gb * uz;
    rec[20 + v] = LRb * idLR;
  }
}

// per face: lambda_F, the flux products at the reconstructed states, then both sides'
// reconstructions reversed into rec [50][ldf] (side 0 rows 0..24, side 1 rows 25..49; on a
// periodic face side 1 is the partner face's side 0, whose state is this face's right state)
template <int SCH>
__global__ void __launch_bounds__(128) k_adj_face2(DevMesh m, DevState s, SpatOpts o,
                                                   const double* __restrict__ lamR, double dt,
                                                   double* __restrict__ rec) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const size_t ld = m.ldc, lf = m.ldf;
  const int c1 = m.fc1[f];
  const bool interior = f < m.nfi;
  const double S = m.fs[f];
  double Fb[5], QL[5], QR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    double a = -(dt / m.cvol[c1]) * lamR[v * ld + c1];
    if (interior) a = a + (dt / m.cvol[m.fc2[f]]) * lamR[v * ld + m.fc2[f]];
    Fb[v] = S * a;
  }
  const int F1 = interior ? f : m.part[f], s1 = interior ? 1 : 0;
  recon(m, s, o, f, 0, QL);
  recon(m, s, o, F1, s1, QR);
  // frozen post-limiter: each side's increment scaled by its owner cell's ratio
  double rL[3] = {1.0, 1.0, 1.0}, rR[3] = {1.0, 1.0, 1.0};
  if (o.postlim != TY_POSTLIM_NONE) {
    const int cR = s1 ? m.fc2[F1] : m.fc1[F1];
#pragma unroll
    for (int k = 0; k < 3; ++k) { rL[k] = s.ratio[k * ld + c1]; rR[k] = s.ratio[k * ld + cR]; }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const int k = v < 2 ? v : 2;
      const double qL = s.prim[v * ld + c1], qR = s.prim[v * ld + cR];
      QL[v] = qL + rL[k] * (QL[v] - qL);
      QR[v] = qR + rR[k] * (QR[v] - qR);
    }
  }
  double QLb[5] = {0, 0, 0, 0, 0}, QRb[5] = {0, 0, 0, 0, 0};
  const double nx = d3(m.fn, m.ldf, f, 0), ny = d3(m.fn, m.ldf, f, 1), nz = d3(m.fn, m.ldf, f, 2);
  if constexpr (SCH == TY_SCH_HLLC) hllc_vjp(o.gamma, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  else if constexpr (SCH == TY_SCH_RUSANOV) rusanov_vjp(o.gamma, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  else roe_vjp(o.gamma, o.entropy_fix, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  double r[25];
  recon_vjp(m, s, o, f, 0, QLb, rL, r);
#pragma unroll
  for (int k = 0; k < 25; ++k) rec[k * lf + f] = r[k];
  recon_vjp(m, s, o, F1, s1, QRb, rR, r);
#pragma unroll
  for (int k = 0; k < 25; ++k) rec[(25 + k) * lf + f] = r[k];
}

// per cell: the reversed reconstructions gathered into the adjoints of q (qg rows 0..4) and
// of the gradient (rows 5..19)
__global__ void __launch_bounds__(kBlock) k_adj_cell2(DevMesh m, const double* __restrict__ rec,
                                                      double* __restrict__ qg) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t lf = m.ldf;
  auto R = [&](int f, int side, int k) { return rec[(25 * side + k) * lf + f]; };
  double q[5] = {0, 0, 0, 0, 0}, g[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) g[k] = 0.0;
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = m.cf[sl * (size_t)m.nci + c];
    if (e < 0) break;
    const int f = e >> 1;
    if ((e & 1) == 0) {
#pragma unroll
      for (int k = 0; k < 5; ++k) q[k] += R(f, 0, k) - R(f, 0, 20 + k);
#pragma unroll
      for (int k = 0; k < 15; ++k) g[k] += R(f, 0, 5 + k);
      if (f < m.nfi) {
#pragma unroll
        for (int k = 0; k < 5; ++k) q[k] -= R(f, 1, 20 + k);
      } else {  // periodic: partner p; its right state is this cell's reconstruction
        const int p = m.part[f];
#pragma unroll
        for (int k = 0; k < 5; ++k) q[k] += R(p, 1, k) - R(p, 1, 20 + k) + R(f, 1, 20 + k) + R(p, 0, 20 + k);
#pragma unroll
        for (int k = 0; k < 15; ++k) g[k] += R(p, 1, 5 + k);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 5; ++k) q[k] += R(f, 1, k) + R(f, 1, 20 + k) + R(f, 0, 20 + k);
#pragma unroll
      for (int k = 0; k < 15; ++k) g[k] += R(f, 1, 5 + k);
    }
  }
  const size_t ld = m.ldc;
#pragma unroll
  for (int k = 0; k < 5; ++k) qg[k * ld + c] = q[k];
#pragma unroll
  for (int k = 0; k < 15; ++k) qg[(5 + k) * ld + c] = g[k];
}

// per cell: the least-squares gradient reversed as a gather (G_c = sum_f w_f,c (q_fc2 - q_fc1),
// periodic neighbours through the partner face), then cons -> prim reversed
__global__ void __launch_bounds__(kBlock) k_adj_cell3(DevMesh m, SpatOpts o, const double* __restrict__ u,
                                                      const double* __restrict__ qg, double* __restrict__ lamU) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t ld = m.ldc, lf = m.ldf;
  double qb[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) qb[v] = qg[v * ld + c];
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = m.cf[sl * (size_t)m.nci + c];
    if (e < 0) break;
    const int f = e >> 1, side = e & 1;
    const double sg = side ? 1.0 : -1.0;
    const double wx = m.lsqw[(3 * side) * lf + f], wy = m.lsqw[(3 * side + 1) * lf + f],
                 wz = m.lsqw[(3 * side + 2) * lf + f];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double t = wx * qg[(5 + 3 * v) * ld + c] + wy * qg[(6 + 3 * v) * ld + c] + wz * qg[(7 + 3 * v) * ld + c];
      qb[v] += sg * t;
    }
    int oc, of, os;
    if (f < m.nfi) { oc = side ? m.fc1[f] : m.fc2[f]; of = f; os = 1 - side; }
    else { of = m.part[f]; oc = m.fc1[of]; os = 0; }  // periodic: the partner cell's gradient sees this cell
    const double sgo = f < m.nfi ? sg : 1.0;
    const double ox = m.lsqw[(3 * os) * lf + of], oy = m.lsqw[(3 * os + 1) * lf + of],
                 oz = m.lsqw[(3 * os + 2) * lf + of];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double t = ox * qg[(5 + 3 * v) * ld + oc] + oy * qg[(6 + 3 * v) * ld + oc] + oz * qg[(7 + 3 * v) * ld + oc];
      qb[v] += sgo * t;
    }
  }
  double U[5], Q[5], Ub[5] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int v = 0; v < 5; ++v) U[v] = u[v * ld + c];
  const double ir = prim_r(o.gamma, U, Q);
  prim_vjp(o.gamma, U, ir, qb, Ub);
#pragma unroll
  for (int v = 0; v < 5; ++v) lamU[v * ld + c] = Ub[v];
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

cudaError_t adjoint_vjp_muscl(const DevMesh& m, const DevState& s, const SpatOpts& o, const double* u,
                              const double* lamR, double dt, double* rec, double* qg, double* lamU, cudaStream_t st) {
  k_prim<<<nblk(m.nci), kBlock, 0, st>>>(m, u, s.prim, o.gamma);
  if (m.ng > 0) k_ghost_prim<<<nblk(m.ng), kBlock, 0, st>>>(m, s.prim, o);
  if (o.postlim != TY_POSTLIM_NONE) {  // gradient and the Barth ratios of the forward residual
    const double klim = o.postlim == TY_POSTLIM_SUPERBARTH ? 1.0 : 0.5;
    if (kFast) {
      if (m.nslot <= 4) k_cell_fast<4, 128><<<(unsigned)((m.nci + 127) / 128), 128, 0, st>>>(m, s, o, klim);
      else k_cell_fast<8, 64><<<(unsigned)((m.nci + 63) / 64), 64, 0, st>>>(m, s, o, klim);
    } else {
      k_grad<<<nblk(m.nci), kBlock, 0, st>>>(m, s);
      k_face_states<<<nblk(m.nf), kBlock, 0, st>>>(m, s, o);
      k_barth<<<nblk(m.nci), kBlock, 0, st>>>(m, s, klim);
    }
  } else {
    k_grad<<<nblk(m.nci), kBlock, 0, st>>>(m, s);
  }
  const unsigned gf = (unsigned)((m.nf + 127) / 128);
  if (o.scheme == TY_SCH_HLLC) k_adj_face2<TY_SCH_HLLC><<<gf, 128, 0, st>>>(m, s, o, lamR, dt, rec);
  else if (o.scheme == TY_SCH_RUSANOV) k_adj_face2<TY_SCH_RUSANOV><<<gf, 128, 0, st>>>(m, s, o, lamR, dt, rec);
  else k_adj_face2<TY_SCH_ROE><<<gf, 128, 0, st>>>(m, s, o, lamR, dt, rec);
  k_adj_cell2<<<nblk(m.nci), kBlock, 0, st>>>(m, rec, qg);
  k_adj_cell3<<<nblk(m.nci), kBlock, 0, st>>>(m, o, u, qg, lamU);
  return cudaGetLastError();
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
