// Device state of the heat-conduction (KDIF) path of one ty_mesh handle, and the launchers
// of its kernels.  Temperature lives per cell (ghosts included); the implicit step solves
// the symmetrised system diag(V/dt) A dU = sum(+-F S) (U = Cp T) by conjugate gradients.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "devmesh.hpp"

namespace tyk {

struct KdifState {
  bool ready = false;
  int scheme = 2;               // ty_kdif_flux
  double cp = 1.0;
  double* k = nullptr;          // [ldc] conductivity, ghosts: the inside (or periodic source) cell's
  int* fkind = nullptr;         // [nf] ty_kdif_bc (0 interior, periodic from the mesh)
  double* fval = nullptr;       // [nf] wall temperature or imposed flux
  const double* kgeo = nullptr; // [6][ldf] per face: dHL, dHR (normalised), C_R - C_L (3), (d.n)/|d|^2
  double* T = nullptr;          // [ldc]
  double* grad = nullptr;       // [3][ldc]
  double* flux = nullptr;       // [nf] F S
  double* jac = nullptr;        // [nf] J_R S (0 on imposed-flux faces)
  double* diag = nullptr;       // [nci]
  double* bal = nullptr;        // [nci] sum(+-F S)
  double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;  // [nci] CG, FP64
  float *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *q32 = nullptr, *x32 = nullptr;  // FP32 CG
  float *diag32 = nullptr, *jac32 = nullptr;
  double* part = nullptr;       // [4][kRedBlocks]
  double* scal = nullptr;       // [16] device scalars
  double* pinned = nullptr;     // host mirror of scal
  int* cfo = nullptr;           // [nslot][nci] faces in ascending order (diagonal, mat-vec)
  int* cfon = nullptr;
  // fused conjugate gradients: the symmetrised matrix in difference form,
  //   (S x)_c = m_c x_c + sum_sl a[sl][c] (x_c - x[nb[sl][c]]),
  // m_c = V_c/dt + the conductances of the cell's boundary faces, a = the conductance
  // -J_R S of each interior face (0 with nb = c in unused slots)
  double* ell_m = nullptr;      // [nci]
  double* ell_a = nullptr;      // [nslot][nci]
  float* ell_a32 = nullptr;     // [nslot][nci] the same conductances in FP32
  int* ell_nb = nullptr;        // [nslot][nci]
  double* dinv = nullptr;       // [nci] 1 / diagonal (Jacobi)
  double* s = nullptr;          // [nci] S p (the single-reduction recurrence)
  unsigned* count = nullptr;    // [2] finished blocks of the two fused kernels (last block reduces)
};

#define TY_DECLARE_KDIF(NS)                                                                          \
  namespace NS {                                                                                     \
  cudaError_t kdif_residual(const DevMesh& m, const KdifState& k, double dt, cudaStream_t st);         \
  cudaError_t kdif_assemble(const DevMesh& m, const KdifState& k, double dt, int want32, cudaStream_t st);\
  cudaError_t kdif_matvec(const DevMesh& m, const KdifState& k, const double* x, double* y,           \
                          cudaStream_t st);                                                           \
  cudaError_t kdif_cg_start(const DevMesh& m, const KdifState& k, int f32, cudaStream_t st);          \
  cudaError_t kdif_ell_build(const DevMesh& m, const KdifState& k, double dt, cudaStream_t st);         \
  cudaError_t kdif_fcg_a(const DevMesh& m, const KdifState& k, int first, cudaStream_t st);              \
  cudaError_t kdif_fcg_b(const DevMesh& m, const KdifState& k, int first, int f32, cudaStream_t st);     \
  cudaError_t kdif_fcg_replace(const DevMesh& m, const KdifState& k, cudaStream_t st);                  \
  cudaError_t kdif_cg_iter(const DevMesh& m, const KdifState& k, int f32, cudaStream_t st);           \
  cudaError_t kdif_residual64(const DevMesh& m, const KdifState& k, cudaStream_t st);                 \
  cudaError_t kdif_refine(const DevMesh& m, const KdifState& k, cudaStream_t st);                     \
  cudaError_t kdif_update_T(const DevMesh& m, const KdifState& k, cudaStream_t st);                   \
  }

TY_DECLARE_KDIF(kexact)
TY_DECLARE_KDIF(kfast)

}  // namespace tyk
