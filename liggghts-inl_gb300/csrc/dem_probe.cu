// FP64 FMA throughput probe (diagnostic entry point dem_measure_fp64_peak).
// Eight independent DFMA chains per thread keep the FP64 pipe busy; the
// result is written so that nothing is optimised away.  Grid: 8 blocks of
// 256 threads per SM.
#include <cuda_runtime.h>

#include "../../include/liggghts_gb300.h"

namespace {

__global__ void __launch_bounds__(256) k_dfma_probe(double *out, int iters, double b, double c) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int dem_measure_fp64_peak(double *tflops) {
  if (!tflops) return DEM_ERR_BAD_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEM_ERR_NO_DEVICE;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return DEM_ERR_CUDA;
  const int blocks = nsm * 8, threads = 256, iters = 4096;
  double *out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return DEM_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_probe<<<blocks, threads>>>(out, iters, 0.9999999, 1e-7);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; rep++) {
    cudaEventRecord(e0);
    k_dfma_probe<<<blocks, threads>>>(out, iters, 0.9999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return DEM_ERR_CUDA;
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return DEM_OK;
}
