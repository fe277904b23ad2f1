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
      if (m.nslot <= 4) k_cell_fast<4, 128><<<(unsigned)((m.nci + 127) / 128), 128, 0, st>>>(m, s, o, klim, true);
      else k_cell_fast<8, 64><<<(unsigned)((m.nci + 63) / 64), 64, 0, st>>>(m, s, o, klim, true);
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


#if TY_FAST
// ---- fast-mode second-order adjoint.  Same mathematics as adjoint_vjp_muscl, arranged for
// the FP64 pipe and for whole-sector gathers: records in array-of-structures layout (a
// gather over random neighbours reads whole 32-byte sectors, where the structure-of-arrays
// fields used above read 8 bytes of each), per-slot weight tables read coalesced, Newton-
// Raphson reciprocals and the precomputed 1/V, 1/dLR and reconstruction weights.
//
// cell record, 32 doubles per interior cell: q (5), G (15: grad rho, grad p, du_i/dx_j row i),
// the frozen Barth ratios (3; 1 without a post-limiter), dt/V lambda_R (5), padding (4)
constexpr int kAdjCell = 32;
// face record, 44 doubles per face: the gradient adjoints that go to fc1 (15 + pad) and to
// the cell whose reconstruction is the face's right state (fc2, or on a periodic face the
// partner face's inside cell) (15 + pad), then the q adjoints of the two (5 + 5, pad 2)
constexpr int kAdjFace = 44;

// the cell records; without a post-limiter the least-squares gradient is computed here,
// grad = Wown q_c + sum over slots (+-A^-1 d) q_nb, from the per-slot weight tables (read
// coalesced) instead of a separate gradient kernel
__global__ void __launch_bounds__(kBlock) k_adj_pack(DevMesh m, DevState s, bool post, const double* __restrict__ lamR,
                                                     int ldR, double dt, const double* __restrict__ wtab,
                                                     double* __restrict__ crec) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t ld = m.ldc, n = m.nci;
  double r[kAdjCell];
#pragma unroll
  for (int v = 0; v < 5; ++v) r[v] = s.prim[v * ld + c];
  if (post) {  // gradient and ratios of the forward kernel
#pragma unroll
    for (int k = 0; k < 15; ++k) r[5 + k] = s.grad[k * ld + c];
#pragma unroll
    for (int k = 0; k < 3; ++k) r[20 + k] = s.ratio[k * ld + c];
  } else {
    // grad = sum (+-w)(q_nb - q_c) = sum (+-w) q_nb + Wown q_c (Wown = -sum (+-w))
    const double wx = wtab[c], wy = wtab[n + c], wz = wtab[2 * n + c];
#pragma unroll
    for (int v = 0; v < 5; ++v) { r[5 + 3 * v] = wx * r[v]; r[6 + 3 * v] = wy * r[v]; r[7 + 3 * v] = wz * r[v]; }
    for (int sl = 0; sl < m.nslot; ++sl) {
      const int nb = m.cfn[sl * n + c];
      if (m.cf[sl * n + c] < 0) break;
      const double* w = wtab + (3 + 3 * (size_t)sl) * n + c;  // own-side weights of the slot
      const double ox = w[0], oy = w[n], oz = w[2 * n];
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double q = s.prim[v * ld + nb];
        r[5 + 3 * v] = fma(q, ox, r[5 + 3 * v]);
        r[6 + 3 * v] = fma(q, oy, r[6 + 3 * v]);
        r[7 + 3 * v] = fma(q, oz, r[7 + 3 * v]);
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) r[20 + k] = 1.0;
  }
  const double w = dt * m.invV[c];
#pragma unroll
  for (int v = 0; v < 5; ++v) r[23 + v] = w * lamR[(size_t)v * ldR + c];
#pragma unroll
  for (int k = 28; k < kAdjCell; ++k) r[k] = 0.0;
  double2* out = reinterpret_cast<double2*>(crec + (size_t)c * kAdjCell);
#pragma unroll
  for (int k = 0; k < kAdjCell / 2; ++k) out[k] = make_double2(r[2 * k], r[2 * k + 1]);
}

// One side of a face: the owner's record O, the other cell's record N, the face F whose
// geometry the reconstruction uses (the face itself, or the partner face of a periodic face)
// and the side of F the owner is on (0: fc1, 1: fc2).  LR = (q_fc2(F) - q_fc1(F)) / dLR =
// (q_N - q_O) / dLR on side 0 and (q_O - q_N) / dLR on side 1.
struct AdjSide {
  const double* O;
  const double* N;
  int F, side;
};

// forward reconstruction of one side (MUSCL / MUSCL-UNS, no limiter or van Albada), the frozen
// ratio r applied to the increment:
//   q = q_O + r (G . CF + sg (u . CF)),  g = G . u,  LR = (q_N - q_O) idLR (idLR signed by side),
//   sg = phi(2g - LR, LR) - g (MUSCL) or phi(g, LR) - g (MUSCL-UNS), phi(a, b) = a b (a + b) /
//   (a^2 + b^2) where a b > 0, else 0 (van Albada);
// with van Albada it also returns the derivatives the reverse needs, cg = dq/dg and
// cq = dq/d(q_N - q_O), so that the reverse does not recompute the limiter.  No limiter: the
// increment is G . w + (q_N - q_O) k with the precomputed weights (recw).
__device__ void adj_recon_f(const DevMesh& m, const SpatOpts& o, const AdjSide& sd, double q[5], double cg[5],
                            double cq[5]) {
  const size_t lf = m.ldf;
  const int F = sd.F;
  const double* __restrict__ O = sd.O;
  const double* __restrict__ N = sd.N;
  if (o.limiter == TY_LIM_NONE) {
    const double* w = m.recw + (4 * sd.side) * lf + F;
    const double wx = w[0], wy = w[lf], wz = w[2 * lf], k = w[3 * lf];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double inc = O[5 + 3 * v] * wx + O[6 + 3 * v] * wy + O[7 + 3 * v] * wz + (N[v] - O[v]) * k;
      q[v] = O[v] + O[20 + (v < 2 ? v : 2)] * inc;
    }
    return;
  }
  // G . CF - g (u . CF) = G . w with w = CF - (u . CF) u, the no-limiter weights (recw)
  const bool uns = o.highres == TY_HRES_MUSCLUNS;
  const double ux = m.uLR[F], uy = m.uLR[lf + F], uz = m.uLR[2 * lf + F];
  const double* w = m.recw + (4 * sd.side) * lf + F;
  const double wx = w[0], wy = w[lf], wz = w[2 * lf];
  const double* CF = sd.side ? m.RF : m.LF;
  const double uc = ux * CF[F] + uy * CF[lf + F] + uz * CF[2 * lf + F];
  const double idLR = sd.side ? -m.invdLR[F] : m.invdLR[F];
  double ruc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) ruc[k] = O[20 + k] * uc;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double gx = O[5 + 3 * v], gy = O[6 + 3 * v], gz = O[7 + 3 * v];
    const double g = gx * ux + gy * uy + gz * uz;
    const double LR = (N[v] - O[v]) * idLR;
    const double a = uns ? g : 2.0 * g - LR, b = LR;
    const double ab = a * b;
    const double rc = ruc[v < 2 ? v : 2];
    // phi = a b (a + b) / D, D = a^2 + b^2; dphi/da = b^2 (b^2 - a^2 + 2ab) / D^2,
    // dphi/db = a^2 (a^2 - b^2 + 2ab) / D^2
    double phi = 0.0, cgv = -rc, cqv = 0.0;
    if (ab > 0.0) {
      const double a2 = a * a, b2 = b * b, iD = rcp_nr(a2 + b2);
      phi = ab * (a + b) * iD;
      const double dl = b2 - a2;
      const double X = b2 * fma(2.0, ab, dl), Y = a2 * fma(2.0, ab, -dl);  // D^2 dphi/da, D^2 dphi/db
      const double k1 = rc * (iD * iD);
      cgv = uns ? fma(X, k1, -rc) : fma(2.0 * X, k1, -rc);
      cqv = (uns ? Y : Y - X) * k1 * idLR;
    }
    const double inc = fma(phi, uc, gx * wx + gy * wy + gz * wz);
    q[v] = fma(O[20 + (v < 2 ? v : 2)], inc, O[v]);
    cg[v] = cgv;
    cq[v] = cqv;
  }
}

// reverse of adj_recon_f: Qb -> adjoints of the owner's q (own), of the other cell's q (oth)
// and of the owner's gradient (G)
__device__ void adj_recon_b(const DevMesh& m, const SpatOpts& o, const AdjSide& sd, const double Qb[5],
                            const double cg[5], const double cq[5], double own[5], double oth[5], double G[15]) {
  const size_t lf = m.ldf;
  const int F = sd.F;
  const double* __restrict__ O = sd.O;
  if (o.limiter == TY_LIM_NONE) {
    const double* w = m.recw + (4 * sd.side) * lf + F;
    const double wx = w[0], wy = w[lf], wz = w[2 * lf], k = w[3 * lf];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double d = O[20 + (v < 2 ? v : 2)] * Qb[v];
      own[v] = Qb[v] - d * k;
      oth[v] = d * k;
      G[3 * v] = d * wx; G[3 * v + 1] = d * wy; G[3 * v + 2] = d * wz;
    }
    return;
  }
  const double ux = m.uLR[F], uy = m.uLR[lf + F], uz = m.uLR[2 * lf + F];
  const double* CF = sd.side ? m.RF : m.LF;
  const double cx = CF[F], cy = CF[lf + F], cz = CF[2 * lf + F];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double db = O[20 + (v < 2 ? v : 2)] * Qb[v], gb = cg[v] * Qb[v], dqb = cq[v] * Qb[v];
    own[v] = Qb[v] - dqb;
    oth[v] = dqb;
    G[3 * v] = db * cx + gb * ux;
    G[3 * v + 1] = db * cy + gb * uy;
    G[3 * v + 2] = db * cz + gb * uz;
  }
}

__device__ __forceinline__ void adj_store_g(double* rec, const double G[15]) {
  double2* o = reinterpret_cast<double2*>(rec);
#pragma unroll
  for (int k = 0; k < 7; ++k) o[k] = make_double2(G[2 * k], G[2 * k + 1]);
  o[7] = make_double2(G[14], 0.0);
}

// per face: lambda_F, the flux products at the reconstructed states, both reconstructions
// reversed, summed per destination cell into the face record
template <int SCH>
__device__ __forceinline__ void adj_face2f(const DevMesh& m, const SpatOpts& o, const double* __restrict__ crec,
                                           double* __restrict__ frec, int f) {
  const bool interior = f < m.nfi;
  const int c1 = m.fc1[f];
  const int F1 = interior ? f : m.part[f];
  const int cR = interior ? m.fc2[f] : m.fc1[F1];
  const double* A = crec + (size_t)c1 * kAdjCell;
  const double* B = crec + (size_t)cR * kAdjCell;
  const double S = m.fs[f];
  double Fb[5], QL[5], QR[5], cg0[5], cq0[5], cg1[5], cq1[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) Fb[v] = interior ? S * (B[23 + v] - A[23 + v]) : -S * A[23 + v];
  const AdjSide s0{A, B, f, 0}, s1{B, A, F1, interior ? 1 : 0};
  adj_recon_f(m, o, s0, QL, cg0, cq0);
  adj_recon_f(m, o, s1, QR, cg1, cq1);
  double QLb[5] = {0, 0, 0, 0, 0}, QRb[5] = {0, 0, 0, 0, 0};
  const size_t lf = m.ldf;
  const double nx = m.fn[f], ny = m.fn[lf + f], nz = m.fn[2 * lf + f];
  if constexpr (SCH == TY_SCH_HLLC) hllc_vjp(o.gamma, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  else if constexpr (SCH == TY_SCH_RUSANOV) rusanov_vjp(o.gamma, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  else roe_vjp(o.gamma, o.entropy_fix, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  double* rec = frec + (size_t)f * kAdjFace;
  double own0[5], oth0[5], own1[5], oth1[5], G[15];
  adj_recon_b(m, o, s0, QLb, cg0, cq0, own0, oth0, G);
  adj_store_g(rec, G);
  adj_recon_b(m, o, s1, QRb, cg1, cq1, own1, oth1, G);
  adj_store_g(rec + 16, G);
  // to fc1: its own reconstruction's q adjoint and the right side's adjoint of its q as the
  // other cell; to the right-state cell the converse
  double d[12];
#pragma unroll
  for (int v = 0; v < 5; ++v) { d[v] = own0[v] + oth1[v]; d[5 + v] = own1[v] + oth0[v]; }
  d[10] = 0.0; d[11] = 0.0;
  double2* oq = reinterpret_cast<double2*>(rec + 32);
#pragma unroll
  for (int k = 0; k < 6; ++k) oq[k] = make_double2(d[2 * k], d[2 * k + 1]);
}

template <int SCH>
__global__ void __launch_bounds__(128) k_adj_face2f(DevMesh m, SpatOpts o, const double* __restrict__ crec,
                                                    double* __restrict__ frec) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < m.nf) adj_face2f<SCH>(m, o, crec, frec, f);
}
// Roe's reverse holds more values: three blocks per SM (a few spilled registers) rather than two
__global__ void __launch_bounds__(128, 3) k_adj_face2f_roe(DevMesh m, SpatOpts o, const double* __restrict__ crec,
                                                           double* __restrict__ frec) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < m.nf) adj_face2f<TY_SCH_ROE>(m, o, crec, frec, f);
}

// per cell: the face records gathered (side s of a face: gradient block 16 s, q block 32 + 5 s;
// a periodic face also brings its partner face's right-state block) into the adjoints of the
// cell's q and gradient; the gradient's adjoint is then reversed through the least-squares
// weights: the cell's own term is added to qb [5][ldc], and the term of each neighbour
// (G_c = Wown q_c + sum over slots wo_slot q_nb) is written to ctb [nf][2][5] at the face and
// this cell's side, for the neighbour's gather (k_adj_cell3f).  NS >= nslot: the slot loop is
// unrolled so that every record load is issued before the first is used.
template <int NS>
__global__ void __launch_bounds__(kBlock) k_adj_cell2f(DevMesh m, const double* __restrict__ frec,
                                                       const double* __restrict__ wtab, double* __restrict__ qb,
                                                       double* __restrict__ ctb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t n = m.nci;
  int rf[2 * NS], rs[2 * NS];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int e = sl < m.nslot ? m.cf[sl * n + c] : -1;
    const int f = e >> 1, side = e & 1;
    rf[2 * sl] = e < 0 ? -1 : f;
    rs[2 * sl] = side;
    // periodic face owned by this cell: the partner face's right-state block
    rf[2 * sl + 1] = (e >= 0 && !side && f >= m.nfi) ? m.part[f] : -1;
    rs[2 * sl + 1] = 1;
  }
  double q[5] = {0, 0, 0, 0, 0}, g[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) g[k] = 0.0;
#pragma unroll
  for (int i = 0; i < 2 * NS; ++i) {
    if (rf[i] < 0) continue;
    const double* r = frec + (size_t)rf[i] * kAdjFace;
    const double2* rg = reinterpret_cast<const double2*>(r + 16 * rs[i]);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const double2 t = rg[k];
      g[2 * k] += t.x;
      g[2 * k + 1] += t.y;
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) q[v] += r[32 + 5 * rs[i] + v];
  }
  {
    const double wx = wtab[c], wy = wtab[n + c], wz = wtab[2 * n + c];
#pragma unroll
    for (int v = 0; v < 5; ++v) q[v] += wx * g[3 * v] + wy * g[3 * v + 1] + wz * g[3 * v + 2];
  }
  const size_t ld = m.ldc;
#pragma unroll
  for (int v = 0; v < 5; ++v) qb[v * ld + c] = q[v];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int f = rf[2 * sl];
    if (f < 0) continue;
    const double* w = wtab + (3 + 3 * (size_t)sl) * n + c;
    const double wx = w[0], wy = w[n], wz = w[2 * n];
    double* o = ctb + (size_t)f * 10 + 5 * rs[2 * sl];
#pragma unroll
    for (int v = 0; v < 5; ++v) o[v] = wx * g[3 * v] + wy * g[3 * v + 1] + wz * g[3 * v + 2];
  }
}

// per cell: the neighbours' least-squares terms gathered from ctb (an interior face's other
// side; on a periodic face owned by this cell, the partner face's owner side, whose ghost is
// this cell), then cons -> prim reversed
template <int NS>
__global__ void __launch_bounds__(kBlock) k_adj_cell3f(DevMesh m, SpatOpts o, const double* __restrict__ u,
                                                       const double* __restrict__ qbuf, const double* __restrict__ ctb,
                                                       double* __restrict__ lamU, int ldU) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t ld = m.ldc, n = m.nci;
  int rf[NS];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int e = sl < m.nslot ? m.cf[sl * n + c] : -1;
    const int f = e >> 1, side = e & 1;
    rf[sl] = e < 0 ? -1 : (f < m.nfi ? 10 * f + 5 * (1 - side) : 10 * m.part[f]);
  }
  double qb[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) qb[v] = qbuf[v * ld + c];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    if (rf[sl] < 0) continue;
    const double* r = ctb + rf[sl];
#pragma unroll
    for (int v = 0; v < 5; ++v) qb[v] += r[v];
  }
  double U[5], Q[5], Ub[5] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int v = 0; v < 5; ++v) U[v] = u[v * ld + c];
  const double ir = prim_r(o.gamma, U, Q);
  prim_vjp(o.gamma, U, ir, qb, Ub);
#pragma unroll
  for (int v = 0; v < 5; ++v) lamU[(size_t)v * ldU + c] = Ub[v];
}

// the weight tables of k_adj_pack and k_adj_cell2f (static geometry): Wown [3][nci] = sum over
// the cell's faces of -+ (A^-1 d) of its side, and per slot [3][nci] the cell's own +-(A^-1 d)
// (its gradient is the sum of these times q_nb plus Wown q_c; zero past the last face)
__global__ void __launch_bounds__(kBlock) k_adj_wbuild(DevMesh m, double* __restrict__ wtab) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t n = m.nci, lf = m.ldf;
  double W[3] = {0, 0, 0};
  for (int sl = 0; sl < m.nslot; ++sl) {
    const int e = m.cf[sl * n + c];
    double* wo = wtab + (3 + 3 * (size_t)sl) * n + c;
    if (e < 0) {
      wo[0] = wo[n] = wo[2 * n] = 0.0;
      continue;
    }
    const int f = e >> 1, side = e & 1;
    const double sg = side ? 1.0 : -1.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      W[j] += sg * m.lsqw[(3 * side + j) * lf + f];
      wo[j * n] = -sg * m.lsqw[(3 * side + j) * lf + f];
    }
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) wtab[j * n + c] = W[j];
}

cudaError_t adjoint_weights_fast(const DevMesh& m, double* wtab, cudaStream_t st) {
  k_adj_wbuild<<<nblk(m.nci), kBlock, 0, st>>>(m, wtab);
  return cudaGetLastError();
}

cudaError_t adjoint_vjp_muscl_fast(const DevMesh& m, const DevState& s, const SpatOpts& o, const double* u,
                                   const double* lamR, int ldR, double dt, double* crec, double* frec, double* qbuf,
                                   double* ctb, const double* wtab, double* lamU, int ldU, cudaStream_t st) {
  k_prim<<<nblk(m.nci), kBlock, 0, st>>>(m, u, s.prim, o.gamma);
  if (m.ng > 0) k_ghost_prim<<<nblk(m.ng), kBlock, 0, st>>>(m, s.prim, o);
  const bool post = o.postlim != TY_POSTLIM_NONE;
  if (post) {  // gradient and the Barth ratios of the forward residual
    const double klim = o.postlim == TY_POSTLIM_SUPERBARTH ? 1.0 : 0.5;
    if (m.nslot <= 4) k_cell_fast<4, 128><<<(unsigned)((m.nci + 127) / 128), 128, 0, st>>>(m, s, o, klim, true);
    else k_cell_fast<8, 64><<<(unsigned)((m.nci + 63) / 64), 64, 0, st>>>(m, s, o, klim, true);
  }
  k_adj_pack<<<nblk(m.nci), kBlock, 0, st>>>(m, s, post, lamR, ldR, dt, wtab, crec);
  const unsigned gf = (unsigned)((m.nf + 127) / 128);
  if (o.scheme == TY_SCH_HLLC) k_adj_face2f<TY_SCH_HLLC><<<gf, 128, 0, st>>>(m, o, crec, frec);
  else if (o.scheme == TY_SCH_RUSANOV) k_adj_face2f<TY_SCH_RUSANOV><<<gf, 128, 0, st>>>(m, o, crec, frec);
  else k_adj_face2f_roe<<<gf, 128, 0, st>>>(m, o, crec, frec);
  if (m.nslot <= 4) {
    k_adj_cell2f<4><<<nblk(m.nci), kBlock, 0, st>>>(m, frec, wtab, qbuf, ctb);
    k_adj_cell3f<4><<<nblk(m.nci), kBlock, 0, st>>>(m, o, u, qbuf, ctb, lamU, ldU);
  } else {
    k_adj_cell2f<kMaxSlot><<<nblk(m.nci), kBlock, 0, st>>>(m, frec, wtab, qbuf, ctb);
    k_adj_cell3f<kMaxSlot><<<nblk(m.nci), kBlock, 0, st>>>(m, o, u, qbuf, ctb, lamU, ldU);
  }
  return cudaGetLastError();
}

// ---- fast-mode first-order adjoint: primitive states and dt/V lambda_R packed per cell (one
// cons -> prim per cell instead of one per face side), the face kernel writes the adjoints of
// the two face states, and the cell kernel reverses cons -> prim once per cell.
constexpr int kAdjCell1 = 12;  // q (5), dt/V lambda_R (5), padding (2)

__global__ void __launch_bounds__(kBlock) k_adj_pack1(DevMesh m, SpatOpts o, const double* __restrict__ u,
                                                      const double* __restrict__ lamR, int ldR, double dt,
                                                      double* __restrict__ crec) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t ld = m.ldc;
  double U[5], r[kAdjCell1];
#pragma unroll
  for (int v = 0; v < 5; ++v) U[v] = u[v * ld + c];
  prim_r(o.gamma, U, r);
  const double w = dt * m.invV[c];
#pragma unroll
  for (int v = 0; v < 5; ++v) r[5 + v] = w * lamR[(size_t)v * ldR + c];
  r[10] = 0.0; r[11] = 0.0;
  double2* out = reinterpret_cast<double2*>(crec + (size_t)c * kAdjCell1);
#pragma unroll
  for (int k = 0; k < kAdjCell1 / 2; ++k) out[k] = make_double2(r[2 * k], r[2 * k + 1]);
}

// per face: the adjoints of the left and right face states (10 doubles; the right one is
// folded into the left through the boundary state on a non-periodic boundary face)
template <int SCH>
__global__ void __launch_bounds__(128) k_adj_face1f(DevMesh m, SpatOpts o, const double* __restrict__ crec,
                                                    double* __restrict__ frec) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nf) return;
  const int c1 = m.fc1[f];
  const int kind = f < m.nfi ? TY_BC_INTERIOR : m.fbc[f];
  const bool two = kind == TY_BC_INTERIOR || kind == TY_BC_PERIODIC;
  const int cR = kind == TY_BC_INTERIOR ? m.fc2[f] : (kind == TY_BC_PERIODIC ? m.fc1[m.part[f]] : c1);
  const double* A = crec + (size_t)c1 * kAdjCell1;
  const double* B = crec + (size_t)cR * kAdjCell1;
  const double S = m.fs[f];
  double Fb[5], QL[5], QR[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    Fb[v] = kind == TY_BC_INTERIOR ? S * (B[5 + v] - A[5 + v]) : -S * A[5 + v];
    QL[v] = A[v];
    QR[v] = B[v];
  }
  if (!two) bc_state(m, o, f, kind, QL, QR);
  double QLb[5] = {0, 0, 0, 0, 0}, QRb[5] = {0, 0, 0, 0, 0};
  const size_t lf = m.ldf;
  const double nx = m.fn[f], ny = m.fn[lf + f], nz = m.fn[2 * lf + f];
  if constexpr (SCH == TY_SCH_HLLC) hllc_vjp(o.gamma, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  else if constexpr (SCH == TY_SCH_RUSANOV) rusanov_vjp(o.gamma, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  else roe_vjp(o.gamma, o.entropy_fix, QL, QR, nx, ny, nz, Fb, QLb, QRb);
  if (!two) {
    bc_state_vjp(m, o, f, kind, QRb, QLb);
#pragma unroll
    for (int v = 0; v < 5; ++v) QRb[v] = 0.0;
  }
  double2* out = reinterpret_cast<double2*>(frec + (size_t)f * 10);
  out[0] = make_double2(QLb[0], QLb[1]);
  out[1] = make_double2(QLb[2], QLb[3]);
  out[2] = make_double2(QLb[4], QRb[0]);
  out[3] = make_double2(QRb[1], QRb[2]);
  out[4] = make_double2(QRb[3], QRb[4]);
}

// per cell: the face-state adjoints of its faces (a periodic face also brings its partner's
// right state, which is this cell's), then cons -> prim reversed
template <int NS>
__global__ void __launch_bounds__(kBlock) k_adj_cell1f(DevMesh m, SpatOpts o, const double* __restrict__ u,
                                                       const double* __restrict__ frec, double* __restrict__ lamU,
                                                       int ldU) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.nci) return;
  const size_t n = m.nci, ld = m.ldc;
  int rf[2 * NS], rs[2 * NS];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int e = sl < m.nslot ? m.cf[sl * n + c] : -1;
    const int f = e >> 1, side = e & 1;
    rf[2 * sl] = e < 0 ? -1 : f;
    rs[2 * sl] = side;
    rf[2 * sl + 1] = (e >= 0 && !side && f >= m.nfi && m.fbc[f] == TY_BC_PERIODIC) ? m.part[f] : -1;
    rs[2 * sl + 1] = 1;
  }
  double qb[5] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < 2 * NS; ++i) {
    if (rf[i] < 0) continue;
    const double* r = frec + (size_t)rf[i] * 10 + 5 * rs[i];
#pragma unroll
    for (int v = 0; v < 5; ++v) qb[v] += r[v];
  }
  double U[5], Q[5], Ub[5] = {0, 0, 0, 0, 0};
#pragma unroll
  for (int v = 0; v < 5; ++v) U[v] = u[v * ld + c];
  const double ir = prim_r(o.gamma, U, Q);
  prim_vjp(o.gamma, U, ir, qb, Ub);
#pragma unroll
  for (int v = 0; v < 5; ++v) lamU[(size_t)v * ldU + c] = Ub[v];
}

cudaError_t adjoint_vjp_fast(const DevMesh& m, const SpatOpts& o, const double* u, const double* lamR, int ldR,
                             double dt, double* crec, double* frec, double* lamU, int ldU, cudaStream_t st) {
  k_adj_pack1<<<nblk(m.nci), kBlock, 0, st>>>(m, o, u, lamR, ldR, dt, crec);
  const unsigned gf = (unsigned)((m.nf + 127) / 128);
  if (o.scheme == TY_SCH_HLLC) k_adj_face1f<TY_SCH_HLLC><<<gf, 128, 0, st>>>(m, o, crec, frec);
  else if (o.scheme == TY_SCH_RUSANOV) k_adj_face1f<TY_SCH_RUSANOV><<<gf, 128, 0, st>>>(m, o, crec, frec);
  else k_adj_face1f<TY_SCH_ROE><<<gf, 128, 0, st>>>(m, o, crec, frec);
  if (m.nslot <= 4) k_adj_cell1f<4><<<nblk(m.nci), kBlock, 0, st>>>(m, o, u, frec, lamU, ldU);
  else k_adj_cell1f<kMaxSlot><<<nblk(m.nci), kBlock, 0, st>>>(m, o, u, frec, lamU, ldU);
  return cudaGetLastError();
}
#endif  // TY_FAST

}  // namespace TY_KNS
}  // namespace tyk
