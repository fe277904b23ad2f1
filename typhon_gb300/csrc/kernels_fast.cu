// Fast-mode instantiation of kernels.cuh (fused multiply-add, precomputed weights).
#define TY_KNS kfast
#define TY_FAST 1
#include "kernels.cuh"
#include "implicit.cuh"
#include "kdif.cuh"
#include "adjoint.cuh"

// ty_debug_fastmath: the Newton-Raphson reciprocal, reciprocal square root and square root of
// fastmath.cuh on caller values, so that their error against CUDA's IEEE division and square
// root can be measured.
#include <cuda_runtime.h>

#include "internal.hpp"

namespace {
__global__ void k_fastmath(int which, int n, const double* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = x[i];
  double r;
  switch (which) {
    case 0: r = tyk::rcp_nr(a); break;
    case 1: r = tyk::rsqrt_nr(a); break;
    case 2: r = tyk::sqrt_nr(a); break;
    case 3: r = 1.0 / a; break;        // CUDA's IEEE division
    case 4: r = 1.0 / sqrt(a); break;  // CUDA's IEEE square root and division
    case 5: r = sqrt(a); break;        // CUDA's IEEE square root
    case 6: r = tyk::rcp_seed(a); break;
    default: r = tyk::rsqrt_seed(a); break;
  }
  y[i] = r;
}
}  // namespace

extern "C" int ty_debug_fastmath(int32_t which, int32_t n, const double* x, double* y) {
  if (which < 0 || which > 7 || n < 0 || (n > 0 && (!x || !y))) return TY_ERR_ARG;
  if (n == 0) return TY_OK;
  double *dx = nullptr, *dy = nullptr;
  const size_t bytes = (size_t)n * sizeof(double);
  cudaError_t e = cudaMalloc(&dx, 2 * bytes);
  if (e == cudaSuccess) {
    dy = dx + n;
    e = cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) {
    k_fastmath<<<(unsigned)((n + 255) / 256), 256>>>(which, n, dx, dy);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(y, dy, bytes, cudaMemcpyDeviceToHost);
  if (dx) cudaFree(dx);
  if (e != cudaSuccess) {
    tyi::set_error(std::string("ty_debug_fastmath: ") + cudaGetErrorString(e));
    return TY_ERR_CUDA;
  }
  return TY_OK;
}
