// Reciprocal, reciprocal square root and square root for the fast mode (TY_MODE_FAST).
//
// GB300 issues FP64 at about 2 DFMA per SM per clock, and an IEEE FP64 division or square
// root costs about ten of them, so the fast kernels replace them with one Newton-Raphson
// step of third order in FP64, seeded by the hardware approximations of PTX
// (rcp.approx.ftz.f64 and rsqrt.approx.ftz.f64, which run on the special-function unit, not
// on the FP64 pipe; measured on GB300 to a relative error below 2^-19.9):
//
//   reciprocal of a:        e = 1 - a x,    x <- x (1 + e + e^2)             (3 DFMA)
//   reciprocal square root: e = 1 - a y^2,  y <- y (1 + e/2 + 3 e^2/8)       (5 FP64 ops)
//
// (Newton's iteration for f(x) = 1/x - a, and Halley's / the third-order Householder step
// for f(y) = 1/y^2 - a: the truncated binomial series of (1 - e)^(-1) and (1 - e)^(-1/2)).
// The remaining relative error is about e^3 ~ 2^-59, so the results are within a few units
// in the last place of the correctly rounded values (not always correctly rounded), which
// the fast mode's tolerance absorbs; ty_debug_fastmath measures them against CUDA's IEEE
// division and square root.  Inputs are positive normal numbers (densities, pressures, sums
// of squares): subnormal inputs are flushed to zero by the seeds.
#pragma once
#include <cuda_runtime.h>

namespace tyk {

__device__ __forceinline__ double rcp_seed(double a) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(a));
  return r;
}

__device__ __forceinline__ double rsqrt_seed(double a) {
  double r;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(a));
  return r;
}

// 1/a: one third-order step from the hardware seed (3 DFMA).
__device__ __forceinline__ double rcp_nr(double a) {
  const double x = rcp_seed(a);
  const double e = fma(-a, x, 1.0);
  return fma(x, fma(e, e, e), x);
}

// 1/sqrt(a), a > 0: one third-order step from the hardware seed (5 FP64 operations).
__device__ __forceinline__ double rsqrt_nr(double a) {
  const double y = rsqrt_seed(a);
  const double e = fma(-a * y, y, 1.0);
  return fma(y * e, fma(0.375, e, 0.5), y);
}

// sqrt(a) = a / sqrt(a) for a > 0; 0 for a == 0 (the product would be 0 * inf).
__device__ __forceinline__ double sqrt_nr(double a) {
  return a > 0.0 ? a * rsqrt_nr(a) : 0.0;
}

}  // namespace tyk
