// Fast-mode instantiation of kernels.cuh (fused multiply-add, precomputed weights).
#define TY_KNS kfast
#define TY_FAST 1
#include "kernels.cuh"
#include "implicit.cuh"
#include "kdif.cuh"
#include "adjoint.cuh"
