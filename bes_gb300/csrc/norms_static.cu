// Residual norms for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a framework whose caching allocator has
// already reserved the device memory it will use (a raw cudaMalloc there can fail or
// fragment the pool), or a latency-critical loop in which a cudaMalloc/cudaFree pair would
// synchronise the whole device.  For them bes_residual_norms_static computes the per-variable
// L2 and max norms of a residual with the same two-kernel reduction the explicit iteration
// uses at its last stage, but keeps the per-block partial sums in a fixed array of device
// memory owned by this file instead of in a buffer from cudaMalloc.  The caller passes the
// residual and the output, both already in device memory.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/bes_gb300.h"

namespace {

constexpr int kNormBlock = 256;
// Largest residual this entry point accepts: one block of partial sums per 256 cells.
constexpr int64_t kStaticNormMaxCells = 4194304;                     // 2^22 cells
constexpr int kStaticNormMaxBlocks = (int)(kStaticNormMaxCells / kNormBlock);  // 16384

// Per-block partial sums: [10][blocks] (5 sums of squares, then 5 maxima), 1.25 MiB.  Every
// GPU that loads the library holds this array until the process exits.  Every call overwrites
// it completely before reading it, so nothing needs clearing between calls; calls that overlap
// on the GPU (two streams, or two host threads) share it and race.
__device__ __align__(256) double g_norm_partials[10 * kStaticNormMaxBlocks];

// Device address of g_norm_partials per CUDA context.  The address is a property of the
// context the module is loaded into, not of the device number: a caller that makes its own
// (non-primary) context with the driver API gets the copy of the array in that context.
constexpr int kMaxContexts = 64;
struct ScratchAddress {
  void* context;
  double* partials;
};
ScratchAddress g_scratch[kMaxContexts] = {};
int g_n_scratch = 0;
std::mutex g_setup_mutex;

// cuCtxGetCurrent through the runtime's driver entry point (the library links only cudart).
typedef int (*CtxGetCurrentFn)(void**);
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

__device__ __forceinline__ double wsum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ double wmax(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Same block reduction as the last-stage update of the explicit iteration, reading a
// residual stored cell-major [n][5].
__global__ void __launch_bounds__(kNormBlock) static_norm_partial_kernel(
    const double* __restrict__ R, int64_t n, double* __restrict__ partials) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double r[5] = {0, 0, 0, 0, 0};
  if (c < n)
#pragma unroll
    for (int v = 0; v < 5; ++v) r[v] = R[c * 5 + v];
  __shared__ double sh[10][kNormBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double s = wsum(r[v] * r[v]);
    const double m = wmax(fabs(r[v]));
    if (lane == 0) {
      sh[v][wid] = s;
      sh[5 + v][wid] = m;
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      double x = lane < kNormBlock / 32 ? sh[k][lane] : 0.0;
      x = k < 5 ? wsum(x) : wmax(x);
      if (lane == 0) partials[(int64_t)k * gridDim.x + blockIdx.x] = x;
    }
  }
}

// One block: reduce the partials in a fixed order; out [10] = L2[5], max[5].
__global__ void __launch_bounds__(kNormBlock) static_norm_final_kernel(
    const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
  __shared__ double sh[kNormBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < 10; ++k) {
    double x = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
      const double y = partials[(int64_t)k * nblocks + b];
      x = k < 5 ? x + y : fmax(x, y);
    }
    x = k < 5 ? wsum(x) : wmax(x);
    if (lane == 0) sh[wid] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      x = lane < kNormBlock / 32 ? sh[lane] : 0.0;
      x = k < 5 ? wsum(x) : wmax(x);
      if (lane == 0) out[k] = k < 5 ? sqrt(x) : x;
    }
    __syncthreads();
  }
}

void put_err(char* err, size_t cap, const char* msg) {
  if (err && cap) std::snprintf(err, cap, "%s", msg);
}

}  // namespace

extern "C" int bes_residual_norms_static(const double* residual, int64_t n_cells, double* norms,
                                         void* stream, char* err, size_t err_cap) {
  if (!residual || !norms || n_cells <= 0) {
    put_err(err, err_cap, "residual and norms must be device pointers and n_cells > 0");
    return BES_ERR_INVALID;
  }
  if (n_cells > kStaticNormMaxCells) {
    char buf[160];
    std::snprintf(buf, sizeof(buf),
                  "n_cells = %lld exceeds the fixed scratch of this entry point (at most %lld "
                  "cells); use the context API for larger meshes",
                  (long long)n_cells, (long long)kStaticNormMaxCells);
    put_err(err, err_cap, buf);
    return BES_ERR_INVALID;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    put_err(err, err_cap, "no usable current CUDA device");
    return BES_ERR_CUDA;
  }
  CtxGetCurrentFn get_ctx = ctx_get_current();
  if (!get_ctx) {
    put_err(err, err_cap, "cuCtxGetCurrent is not available from the CUDA driver");
    return BES_ERR_CUDA;
  }
  double* partials = nullptr;
  {
    // First call in a CUDA context: look up the device address of the scratch array once,
    // with that context current.  (The host-side name g_norm_partials is not a device
    // address.)  With no context current yet, the lookup itself makes the device's primary
    // context current, and the address is recorded under that context.
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    void* cur = nullptr;
    if (get_ctx(&cur) != 0) cur = nullptr;
    for (int k = 0; cur && k < g_n_scratch; ++k)
      if (g_scratch[k].context == cur) partials = g_scratch[k].partials;
    if (!partials) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_norm_partials);
      if (e != cudaSuccess || !p) {
        char buf[160];
        std::snprintf(buf, sizeof(buf), "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        put_err(err, err_cap, buf);
        return BES_ERR_CUDA;
      }
      if (!cur && (get_ctx(&cur) != 0 || !cur)) {
        put_err(err, err_cap, "no current CUDA context after the scratch lookup");
        return BES_ERR_CUDA;
      }
      if (g_n_scratch >= kMaxContexts) {
        put_err(err, err_cap, "too many CUDA contexts have used this entry point (at most 64)");
        return BES_ERR_CUDA;
      }
      g_scratch[g_n_scratch++] = {cur, static_cast<double*>(p)};
      partials = static_cast<double*>(p);
    }
  }
  const int nblocks = (int)((n_cells + kNormBlock - 1) / kNormBlock);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  static_norm_partial_kernel<<<nblocks, kNormBlock, 0, s>>>(residual, n_cells, partials);
  static_norm_final_kernel<<<1, kNormBlock, 0, s>>>(partials, nblocks, norms);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "kernel launch: %s", cudaGetErrorString(e));
    put_err(err, err_cap, buf);
    return BES_ERR_CUDA;
  }
  return BES_OK;
}
