// Launchers of the adjoint (vector-Jacobian product) kernels of the residual.
#pragma once
#include <cuda_runtime.h>

#include "devmesh.hpp"

namespace tyk {

#define TY_DECLARE_ADJOINT(NS)                                                                     \
  namespace NS {                                                                                   \
  cudaError_t adjoint_vjp(const DevMesh& m, const SpatOpts& o, const double* u, const double* lamR, \
                          double dt, double* lam_face, double* lamU, cudaStream_t st);               \
  cudaError_t adjoint_vjp_muscl(const DevMesh& m, const DevState& s, const SpatOpts& o, const double* u, \
                                const double* lamR, double dt, double* rec, double* qg, double* lamU,   \
                                cudaStream_t st);                                                      \
  }

TY_DECLARE_ADJOINT(kexact)
TY_DECLARE_ADJOINT(kfast)

// fast mode only: the first- and second-order adjoints on array-of-structures records (lamR
// and lamU in the caller's [5][ld] layout) and the second order's static weight tables
namespace kfast {
cudaError_t adjoint_vjp_fast(const DevMesh& m, const SpatOpts& o, const double* u, const double* lamR, int ldR,
                             double dt, double* crec, double* frec, double* lamU, int ldU, cudaStream_t st);
cudaError_t adjoint_weights_fast(const DevMesh& m, double* wtab, cudaStream_t st);
cudaError_t adjoint_vjp_muscl_fast(const DevMesh& m, const DevState& s, const SpatOpts& o, const double* u,
                                   const double* lamR, int ldR, double dt, double* crec, double* frec, double* qbuf,
                                   double* ctb, const double* wtab, double* lamU, int ldU, cudaStream_t st);
}

}  // namespace tyk
