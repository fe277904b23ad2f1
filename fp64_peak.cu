// FP64 and FP32 arithmetic throughput probe (bench.py reports its DFMA rate as the FP64 peak).
// Every thread writes exactly out[tid]; out holds grid*block elements.
#include <cstdio>
#include <cuda_runtime.h>

template <int ILP>
__global__ void k_dfma(double* out, int iters, double a, double b) {
  double acc[ILP];
#pragma unroll
  for (int i = 0; i < ILP; ++i) acc[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) acc[i] = fma(acc[i], a, b);
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < ILP; ++i) s += acc[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <int ILP>
__global__ void k_ffma(float* out, int iters, float a, float b) {
  float acc[ILP];
#pragma unroll
  for (int i = 0; i < ILP; ++i) acc[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) acc[i] = fmaf(acc[i], a, b);
  }
  float s = 0;
#pragma unroll
  for (int i = 0; i < ILP; ++i) s += acc[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <int ILP>
__global__ void k_ddiv(double* out, int iters, double a) {
  double acc[ILP];
#pragma unroll
  for (int i = 0; i < ILP; ++i) acc[i] = 1.0 + threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) acc[i] = a / acc[i] + 1.0;
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < ILP; ++i) s += acc[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <int ILP>
__global__ void k_dsqrt(double* out, int iters) {
  double acc[ILP];
#pragma unroll
  for (int i = 0; i < ILP; ++i) acc[i] = 2.0 + threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < ILP; ++i) acc[i] = sqrt(acc[i]) + 1.5;
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < ILP; ++i) s += acc[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int main() {
  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, 0);
  printf("device %s SMs %d cc %d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
  const int nsm = p.multiProcessorCount;
  const int block = 256, grid = nsm * 8;
  const size_t n = (size_t)grid * block;
  double* d; float* f;
  cudaMalloc(&d, n * sizeof(double));
  cudaMalloc(&f, n * sizeof(float));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  const int ILP = 8;
  // warm
  k_dfma<ILP><<<grid, block>>>(d, 100, 0.999, 1e-3);
  cudaDeviceSynchronize();
  {
    int iters = 2000;
    cudaEventRecord(e0);
    k_dfma<ILP><<<grid, block>>>(d, iters, 0.999, 1e-3);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)n * iters * ILP;
    printf("DFMA: %.3f ms, %.3f TFMA/s = %.3f TFLOP/s\n", ms, ops / ms * 1e-9, 2 * ops / ms * 1e-9);
  }
  {
    int iters = 20000;
    k_ffma<ILP><<<grid, block>>>(f, 100, 0.999f, 1e-3f);
    cudaEventRecord(e0);
    k_ffma<ILP><<<grid, block>>>(f, iters, 0.999f, 1e-3f);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)n * iters * ILP;
    printf("FFMA: %.3f ms, %.3f TFMA/s = %.3f TFLOP/s\n", ms, ops / ms * 1e-9, 2 * ops / ms * 1e-9);
  }
  {
    int iters = 200;
    k_ddiv<ILP><<<grid, block>>>(d, 10, 3.0);
    cudaEventRecord(e0);
    k_ddiv<ILP><<<grid, block>>>(d, iters, 3.0);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)n * iters * ILP;
    printf("DDIV(+add): %.3f ms, %.3f Gdiv/s\n", ms, ops / ms * 1e-6);
  }
  {
    int iters = 200;
    k_dsqrt<ILP><<<grid, block>>>(d, 10);
    cudaEventRecord(e0);
    k_dsqrt<ILP><<<grid, block>>>(d, iters);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)n * iters * ILP;
    printf("DSQRT(+add): %.3f ms, %.3f Gsqrt/s\n", ms, ops / ms * 1e-6);
  }
  cudaError_t err = cudaGetLastError();
  printf("status %s\n", cudaGetErrorString(err));
  return err == cudaSuccess ? 0 : 1;
}
