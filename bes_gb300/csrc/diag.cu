// FP64 arithmetic rate of the current device, the denominator of the explicit kernels'
// roofline: those kernels do about one FP64 flop per byte they move, several times the ridge
// point of a GPU whose FP64 rate is a small fraction of its FP32 rate, so they are bound by
// the FP64 pipe, not by HBM.  No counterpart in the reference (a CPU code).
#include <cuda_runtime.h>

#include "../../include/bes_gb300.h"

namespace {

constexpr int kChains = 8;      // independent FMA chains per thread
constexpr int kIters = 4096;    // FMAs per chain

__global__ void __launch_bounds__(256) fp64_fma_kernel(double seed, double* __restrict__ sink) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = seed + threadIdx.x * 1e-9 + k * 1e-7;
  const double a = 0.999999999, b = 1e-12;
#pragma unroll 4
  for (int i = 0; i < kIters; ++i)
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], a, b);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  if (s == 12345.678) sink[blockIdx.x] = s;  // never true: keeps the chains live
}

}  // namespace

extern "C" int bes_fp64_fma_rate(double* fma_per_s) {
  if (!fma_per_s) return BES_ERR_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return BES_ERR_CUDA;
  const int blocks = sms * 8;
  double* sink = nullptr;
  if (cudaMalloc(&sink, blocks * sizeof(double)) != cudaSuccess) return BES_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp64_fma_kernel<<<blocks, 256>>>(1.0, sink);  // warm-up
  cudaEventRecord(e0);
  const int reps = 5;
  for (int r = 0; r < reps; ++r) fp64_fma_kernel<<<blocks, 256>>>(1.0 + r, sink);
  cudaEventRecord(e1);
  const cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess || ms <= 0.0f) return BES_ERR_CUDA;
  *fma_per_s = (double)reps * blocks * 256.0 * kChains * kIters / (ms * 1e-3);
  return BES_OK;
}
