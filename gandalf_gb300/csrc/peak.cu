// Fused multiply-add throughput probe (roofline denominators for the pair loops).
#include <cuda_runtime.h>

#include "../../include/gsph_gb300.h"

namespace {

template <typename T>
__global__ void k_fma_loop(T* out, int iters, T a, T b) {
  // 8 independent chains per thread keep the pipe busy; the result is stored so the
  // loop cannot be removed.
  T x[8];
#pragma unroll
  for (int q = 0; q < 8; q++) x[q] = (T) (threadIdx.x + q);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int q = 0; q < 8; q++) x[q] = x[q] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) s += x[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
double run(int device, int iters) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return -1.0;
  const int block = 256;
  const int grid = prop.multiProcessorCount * 8;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * (size_t) grid * block) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_loop<T><<<grid, block>>>(out, iters / 8, (T) 0.999999, (T) 1e-7);   // warm-up
  cudaEventRecord(e0);
  k_fma_loop<T><<<grid, block>>>(out, iters, (T) 0.999999, (T) 1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * (double) iters * grid * block;
  return ms > 0.0f ? flops / (ms * 1e-3) / 1e9 : -1.0;
}

}  // namespace

extern "C" double gsph_fma_peak_gflops(int32_t device, int32_t fp64) {
  if (cudaSetDevice(device) != cudaSuccess) return -1.0;
  return fp64 ? run<double>(device, 4096) : run<float>(device, 65536);
}
