// ty_timestep_static: the global stability time step without any device allocation.
//
// Why it exists.  Some callers cannot let a library call cudaMalloc: a host code that owns
// every byte of device memory through its own pool or allocator and forbids allocations
// behind its back, a long-running solver loop that must not allocate between steps, or a
// Fortran program that hands over device arrays it manages itself.  ty_timestep needs a
// ty_mesh handle, and creating one allocates.  This entry point takes the state and the
// geometric factors as device pointers the caller already owns, and keeps its only scratch
// memory — one partial minimum per thread block and an error word — in a file-scope
// __device__ array compiled into the library.  It has no counterpart in the reference.
//
// Scratch: one array of kMaxBlocks + 2 64-bit words (about 128 KiB): a partial minimum per
// thread block, the result, and an error word (code, cell).  It is resident on every GPU
// that loads the library until the process exits.  Every call shares this array and it
// keeps the contents of the previous call; the error word is cleared at the start of each
// call, the partial minima and the result are overwritten by every call.  Two calls that
// overlap on the GPU (different streams, or different host threads on the same device)
// race on the array and give undefined results: serialise them.
//
// Module loading.  With CUDA's lazy loading (the default), the first call in a CUDA context
// makes the driver load this library's module, and that load allocates device memory for the
// code and for the array.  Later calls in the same context allocate nothing.  A caller that
// must not allocate during its run makes one call at set-up (it also has to come before any
// stream capture).
//
// The per-cell formula is calc_ns_timestep's (SOURCE/EQNS/calc_ns_timestep.f90:52-103):
// dt_c = CFL*2*V_c / sum_f S_f / (|u| + a), each operation rounded separately (this file is
// compiled with -fmad=false), then the minimum over cells (calc_zonetimestep.f90:95).
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "../../include/typhon_gpu.h"
#include "internal.hpp"

namespace {

constexpr int kBlock = 256;
constexpr int kMaxBlocks = 16384;  // cells per call at most kBlock * kMaxBlocks = 4,194,304

constexpr int kResult = kMaxBlocks;      // slot of the result
constexpr int kErr = kMaxBlocks + 1;     // slot of the error word: int code, int cell
static __device__ __align__(256) unsigned long long g_scratch[kMaxBlocks + 2];

__global__ void __launch_bounds__(kBlock) k_dt_blockmin(int n, const double* __restrict__ cons, int ld,
                                                        const double* __restrict__ vol,
                                                        const double* __restrict__ sums, double gamma, double cfl,
                                                        unsigned long long* __restrict__ blockmin, int* err) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long b = 0x7fefffffffffffffull;  // bit pattern of the largest finite double
  if (c < n) {
    const double gg1 = gamma * (gamma - 1.0);
    double d = cfl * 2.0 * vol[c] / sums[c];
    const double rho = cons[c], rhoE = cons[(size_t)ld + c];
    const double mx = cons[2 * (size_t)ld + c], my = cons[3 * (size_t)ld + c], mz = cons[4 * (size_t)ld + c];
    const double irho = 1.0 / rho;
    const double rv2 = mx * mx + my * my + mz * mz;
    const double a2 = (rhoE - 0.5 * rv2 * irho) * gg1 * irho;
    if (!(a2 > 0.0)) {
      if (atomicCAS(err, 0, TY_ERR_NEGENERGY) == 0) err[1] = c;
    } else {
      d = d / (sqrt(rv2) * irho + sqrt(a2));
      if (!(d > 0.0)) {
        if (atomicCAS(err, 0, TY_ERR_NANDT) == 0) err[1] = c;
      } else {
        b = (unsigned long long)__double_as_longlong(d);  // positive doubles order like their bits
      }
    }
  }
  __shared__ unsigned long long smin[kBlock / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
    b = t < b ? t : b;
  }
  if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    b = threadIdx.x < kBlock / 32 ? smin[threadIdx.x] : 0x7fefffffffffffffull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
      b = t < b ? t : b;
    }
    if (threadIdx.x == 0) blockmin[blockIdx.x] = b;
  }
}

__global__ void __launch_bounds__(kBlock) k_dt_final(int nblocks, const unsigned long long* __restrict__ blockmin,
                                                     double* __restrict__ out) {
  unsigned long long b = 0x7fefffffffffffffull;
  for (int i = threadIdx.x; i < nblocks; i += kBlock) {
    const unsigned long long t = blockmin[i];
    b = t < b ? t : b;
  }
  __shared__ unsigned long long smin[kBlock / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
    b = t < b ? t : b;
  }
  if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x < 32) {
    b = threadIdx.x < kBlock / 32 ? smin[threadIdx.x] : 0x7fefffffffffffffull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_down_sync(0xffffffffu, b, o);
      b = t < b ? t : b;
    }
    if (threadIdx.x == 0) *out = __longlong_as_double((long long)b);
  }
}

// Device address of the scratch array in the CUDA context that is current on this thread.
// In host code the name g_scratch is only a host-side stand-in, never a device address.  The
// address belongs to the context that loaded the library's module, not to the device number:
// after cudaDeviceReset, or when the caller makes another context current on the same
// device, an address kept from an earlier call would point into freed or foreign memory.  So
// it is looked up on every call; cudaGetSymbolAddress allocates nothing once the module is
// loaded in the context.
int scratch_in_current_context(unsigned long long** scratch) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) {
    tyi::set_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return TY_ERR_CUDA;
  }
  *scratch = static_cast<unsigned long long*>(p);
  return TY_OK;
}

}  // namespace

extern "C" int ty_timestep_static(int32_t ncell, const double* cons, int32_t ld, const double* volume,
                                  const double* sum_surface, double gamma, double cfl, void* stream,
                                  double* dt_out) {
  if (ncell <= 0 || ld < ncell || !cons || !volume || !sum_surface || !dt_out || !(gamma > 1.0) || !(cfl > 0.0)) {
    tyi::set_error("ty_timestep_static: invalid argument");
    return TY_ERR_ARG;
  }
  const long long nblocks = ((long long)ncell + kBlock - 1) / kBlock;
  if (nblocks > kMaxBlocks) {
    tyi::set_error("ty_timestep_static: " + std::to_string(ncell) + " cells exceed the static scratch limit of " +
                   std::to_string((long long)kBlock * kMaxBlocks) + " cells");
    return TY_ERR_ARG;
  }
  unsigned long long* scratch = nullptr;
  int rc = scratch_in_current_context(&scratch);
  if (rc != TY_OK) return rc;
  unsigned long long* blockmin = scratch;
  int* err = reinterpret_cast<int*>(scratch + kErr);
  double* dres = reinterpret_cast<double*>(scratch + kResult);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(err, 0, 2 * sizeof(int), st);
  if (e == cudaSuccess) {
    k_dt_blockmin<<<(unsigned)nblocks, kBlock, 0, st>>>(ncell, cons, ld, volume, sum_surface, gamma, cfl, blockmin,
                                                        err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    k_dt_final<<<1, kBlock, 0, st>>>((int)nblocks, blockmin, dres);
    e = cudaGetLastError();
  }
  double dt = 0.0;
  int herr[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&dt, dres, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(herr, err, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    tyi::set_error(std::string("ty_timestep_static: ") + cudaGetErrorString(e));
    return TY_ERR_CUDA;
  }
  if (herr[0] != 0) {
    tyi::set_error(std::string(ty_error_string(herr[0])) + " at cell " + std::to_string(herr[1]));
    return herr[0];
  }
  *dt_out = dt;
  return TY_OK;
}
