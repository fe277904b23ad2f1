// Launchers of the adjoint (vector-Jacobian product) kernels of the first-order residual.
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

}  // namespace tyk
