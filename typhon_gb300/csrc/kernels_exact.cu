// Exact-mode instantiation of kernels.cuh.  Compiled with -fmad=false: every FP64 multiply
// and add is rounded separately, in the order Typhon's Fortran evaluates them.
#define TY_KNS kexact
#define TY_FAST 0
#include "kernels.cuh"
#include "implicit.cuh"
#include "kdif.cuh"
#include "adjoint.cuh"
