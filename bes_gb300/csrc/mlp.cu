// Learned warm start: a FiLM-conditioned coordinate MLP that predicts the converged flow field
// of a freestream condition from the solutions the solver produced for other conditions.
// There is no counterpart in the reference (it always starts from the freestream,
// Solver::setUniversalInitialCondition, include/Solver.hpp:71); the solver still converges
// from the predicted field and judges convergence, and a condition whose prediction is not
// physical (rho <= 0 or p <= 0 in some cell) falls back to the freestream.
//
// Network (the oracle's oracle/mlp_oracle.py restates it in FP64):
//   features  cell centroid x scaled to [-1, 1]^3 by the centroids' bounding box;
//             [sin(pi 2^k x_a), cos(pi 2^k x_a)], k = 0..7, at columns 16a + 2k (+1), x at
//             48..50, zeros up to 64;
//   condition c = (Mach vector - mean) / std over the training conditions;
//   4 hidden layers of width 256: z = h W^T + b; [gamma, beta] = c F^T + g;
//             y = z (1 + gamma) + beta; h = silu(y);
//   output    o = h W4^T + b4 (5 values) = (U - U_inf(c)) / scale.
// GEMMs run on the fifth-generation tensor cores (tcgen05.mma, BF16 operands, FP32
// accumulation in tensor memory) with BF16 copies of the weights and of the activations that
// feed them; everything else is FP32;
// AdamW keeps FP32 master weights.  All reductions are in a fixed order (no atomics), so a
// run is reproducible bit for bit.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "context.hpp"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int kW = 256;        // hidden width
constexpr int kK0 = 64;        // input features
constexpr int kLayers = 4;     // hidden layers
constexpr int kOut = 5;
constexpr int kRowTile = 128;  // rows (samples) per GEMM tile; batches are multiples of it
constexpr int kChunk = 64;     // rows per partial sum of the column reductions

// ---- parameter layout (flat FP32), the order of oracle/mlp_oracle.py layout() ----------------
struct Layout {
  int64_t W[5], b[5], F[4], g[4], n;
  Layout() {
    int64_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
      const int k = l == 0 ? kK0 : kW;
      W[l] = off; off += (int64_t)kW * k;
      b[l] = off; off += kW;
      F[l] = off; off += 2 * kW * 3;
      g[l] = off; off += 2 * kW;
    }
    W[4] = off; off += kOut * kW;
    b[4] = off; off += kOut;
    n = off;
  }
};

// ---- deterministic hashing (splitmix64) ------------------------------------------------------
__host__ __device__ inline uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ float silu(float y) { return y / (1.0f + __expf(-y)); }
__device__ __forceinline__ float dsilu(float y) {
  const float s = 1.0f / (1.0f + __expf(-y));
  return s * (1.0f + y * (1.0f - s));
}

// ---- tensor-core GEMM (tcgen05, accumulator in tensor memory) ----------------------------------
// C[z][m][n] = sum over k in split z of A(m,k) B(k,n), FP32 out, with
//   A(m,k) = A_T ? A[k*lda + m] : A[m*lda + k]
//   B(k,n) = B_T ? B[k*ldb + n] : B[n*ldb + k]
// M % 128 == 0, N % 64 == 0, k_split % 64 == 0 (checked by the caller).  One CTA of 128
// threads computes a 128 x 64 tile of C: per 64-wide slice of k, all threads stage the A and B
// slices in shared memory as K-major 8x8 core matrices (no swizzle; an MN-major operand is
// transposed while it is staged), one thread issues four tcgen05.mma (M 128, N 64, K 16, BF16
// operands, FP32 accumulation in 64 columns of tensor memory) and commits them to an
// mbarrier; after the last slice each warp reads its 32 accumulator rows back with
// tcgen05.ld.  Every wait on the mbarrier gives up after two seconds and sets *err.
constexpr int GBM = 128, GBN = 64, GBK = 64;
constexpr int kCoreBytes = 128;                  // an 8 x 8 core matrix of 16-bit values
constexpr int kSbo = (GBK / 8) * kCoreBytes;     // next 8-row group: one k-slice of cores
constexpr int kLbo = kCoreBytes;                 // next 8 values of k

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major, no swizzle, start address and the two strides
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((kLbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((kSbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of this architecture
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ unsigned long long ns_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// wait for phase `parity` of the mbarrier; false after two seconds
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  const unsigned long long t0 = ns_now();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (ns_now() - t0 > 2000000000ull) return false;
  }
}

// stage a ROWS x 64 (k) slice, rows r0.., k0.., into K-major core matrices: value (r, k) at
// byte (r/8)*kSbo + (k/8)*kLbo + (r%8)*16 + (k%8)*2.  The source is k-contiguous by rows
// (src[r*ld + k]) when !TR, or row-contiguous by k (src[k*ld + r]) when TR.
template <bool TR, int ROWS>
__device__ __forceinline__ void stage_slice(uint8_t* sm, const bf16* __restrict__ src, int ld,
                                            int r0, int k0) {
  if (!TR) {
    // 16-byte pieces: row r, values k..k+7 (one core-matrix row)
    for (int v = threadIdx.x; v < ROWS * (GBK / 8); v += blockDim.x) {
      const int r = v / (GBK / 8), seg = v % (GBK / 8);
      const uint4 x = *reinterpret_cast<const uint4*>(src + (size_t)(r0 + r) * ld + k0 + seg * 8);
      *reinterpret_cast<uint4*>(sm + (r / 8) * kSbo + seg * kLbo + (r % 8) * 16) = x;
    }
  } else {
    // 16-byte pieces along the rows (k fixed, rows r..r+7), scattered to eight core rows
    for (int v = threadIdx.x; v < GBK * (ROWS / 8); v += blockDim.x) {
      const int k = v / (ROWS / 8), rs = v % (ROWS / 8);
      const uint4 x = *reinterpret_cast<const uint4*>(src + (size_t)(k0 + k) * ld + r0 + rs * 8);
      const uint16_t* e = reinterpret_cast<const uint16_t*>(&x);
      uint8_t* base = sm + rs * kSbo + (k / 8) * kLbo + (k % 8) * 2;
#pragma unroll
      for (int q = 0; q < 8; ++q) *reinterpret_cast<uint16_t*>(base + q * 16) = e[q];
    }
  }
}

template <bool A_T, bool B_T>
__global__ void __launch_bounds__(128) gemm_tc_kernel(int M, int N, const bf16* __restrict__ A,
                                                      int lda, const bf16* __restrict__ B,
                                                      int ldb, float* __restrict__ C, int ldc,
                                                      int k_split, int* __restrict__ err) {
  __shared__ __align__(128) uint8_t As[GBM * GBK * 2];
  __shared__ __align__(128) uint8_t Bs[GBN * GBK * 2];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const int k_begin = blockIdx.z * k_split, k_end = k_begin + k_split;
  C += (size_t)blockIdx.z * M * ldc;
  const uint32_t mb = smem_u32(&mbar);
  if (warp == 0) {
    // 64 columns of tensor memory for the 128 x 64 FP32 accumulator
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;\n"
                 :: "r"(smem_u32(&tmem_base)) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(mb) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  constexpr uint32_t idesc = umma_idesc(GBM, GBN);
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = k_begin; k0 < k_end && ok; k0 += GBK) {
    stage_slice<A_T, GBM>(As, A, lda, m0, k0);
    stage_slice<B_T, GBN>(Bs, B, ldb, n0, k0);
    // the staged values (generic proxy) become visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < GBK / 16; ++kk) {
        // K = 16 per instruction: two core matrices along k
        const uint64_t ad = umma_desc(smem_u32(As) + kk * 2 * kLbo);
        const uint64_t bd = umma_desc(smem_u32(Bs) + kk * 2 * kLbo);
        const uint32_t acc = (k0 > k_begin || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
            :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc) : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n"
          :: "r"(mb) : "memory");
    }
    // the slice's products are done before its shared memory is staged again; the verdict
    // is the same for every thread (tcgen05.ld below is a warp-synchronous instruction)
    const int waited = mbar_wait(mb, phase) ? 1 : 0;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    ok = __syncthreads_and(waited) != 0;
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    phase ^= 1;
  }
  if (ok) {
    // each warp reads its 32 rows (tensor-memory lanes 32 w .. 32 w + 31), 16 columns a time
#pragma unroll
    for (int c0 = 0; c0 < GBN; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
          "%13,%14,%15}, [%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
            "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
            "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      float* dst = C + (size_t)(m0 + warp * 32 + lane) * ldc + n0 + c0;
#pragma unroll
      for (int q = 0; q < 16; q += 4)
        *reinterpret_cast<float4*>(dst + q) =
            make_float4(__uint_as_float(r[q]), __uint_as_float(r[q + 1]),
                        __uint_as_float(r[q + 2]), __uint_as_float(r[q + 3]));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;\n" :: "r"(tmem) : "memory");
}

// ---- elementwise and reduction kernels -------------------------------------------------------

// features of every cell: bf16 [n_rows][64] (rows beyond n_cells are zero)
__global__ void encode_kernel(int n_cells, int n_rows, const float* __restrict__ xn,
                              bf16* __restrict__ feat) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_rows) return;
  float f[kK0];
#pragma unroll
  for (int q = 0; q < kK0; ++q) f[q] = 0.0f;
  if (i < n_cells) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double x = xn[i * 3 + a];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const double w = 3.141592653589793 * (double)(1 << k) * x;
        f[16 * a + 2 * k] = (float)sin(w);
        f[16 * a + 2 * k + 1] = (float)cos(w);
      }
      f[48 + a] = (float)x;
    }
  }
#pragma unroll
  for (int q = 0; q < kK0; ++q) feat[(size_t)i * kK0 + q] = __float2bfloat16(f[q]);
}

// Training batch: row r draws (sample, cell) from a hash of (seed, step, r).
__global__ void gather_kernel(int B, uint64_t seed, int64_t step, int n_samples, int n_cells,
                              const bf16* __restrict__ feat, const float* __restrict__ targets,
                              const float* __restrict__ cond, bf16* __restrict__ H0,
                              float* __restrict__ C, float* __restrict__ T) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= B) return;
  const uint64_t h = mix64(seed ^ mix64((uint64_t)step * 0x100000001B3ull + (uint64_t)r));
  const int s = (int)((h & 0xffffffffull) % (uint64_t)n_samples);
  const int c = (int)((h >> 32) % (uint64_t)n_cells);
  const uint4* src = reinterpret_cast<const uint4*>(feat + (size_t)c * kK0);
  uint4* dst = reinterpret_cast<uint4*>(H0 + (size_t)r * kK0);
#pragma unroll
  for (int q = 0; q < kK0 / 8; ++q) dst[q] = src[q];
#pragma unroll
  for (int a = 0; a < 3; ++a) C[r * 3 + a] = cond[s * 3 + a];
#pragma unroll
  for (int v = 0; v < kOut; ++v) T[r * kOut + v] = targets[((size_t)s * n_cells + c) * kOut + v];
}

// FiLM + SiLU forward.  Z [B][256] holds h W^T on entry and z = h W^T + b on exit; Y gets y;
// H gets silu(y) in bf16.
__global__ void film_forward_kernel(int B, float* __restrict__ Z, const float* __restrict__ bias,
                                    const float* __restrict__ F, const float* __restrict__ g,
                                    const float* __restrict__ C, float* __restrict__ Y,
                                    bf16* __restrict__ H) {
  const int j = threadIdx.x;  // column (blockDim 256)
  const float f0 = F[j * 3], f1 = F[j * 3 + 1], f2 = F[j * 3 + 2];
  const float e0 = F[(kW + j) * 3], e1 = F[(kW + j) * 3 + 1], e2 = F[(kW + j) * 3 + 2];
  const float gj = g[j], bj = g[kW + j], bb = bias[j];
  for (int r = blockIdx.x; r < B; r += gridDim.x) {
    const float c0 = C[r * 3], c1 = C[r * 3 + 1], c2 = C[r * 3 + 2];
    const float gam = f0 * c0 + f1 * c1 + f2 * c2 + gj;
    const float bet = e0 * c0 + e1 * c1 + e2 * c2 + bj;
    const size_t q = (size_t)r * kW + j;
    const float z = Z[q] + bb;
    const float y = z * (1.0f + gam) + bet;
    Z[q] = z;
    Y[q] = y;
    H[q] = __float2bfloat16(silu(y));
  }
}

// Output layer, loss and dO: one thread per row; W4 in shared memory.
__global__ void output_forward_kernel(int B, const bf16* __restrict__ H4,
                                      const float* __restrict__ W4, const float* __restrict__ b4,
                                      const float* __restrict__ T, float* __restrict__ O,
                                      float* __restrict__ dO, double* __restrict__ loss_part) {
  __shared__ float w[kOut * kW];
  __shared__ double red[256];
  for (int q = threadIdx.x; q < kOut * kW; q += blockDim.x) w[q] = W4[q];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (r < B) {
    float o[kOut];
#pragma unroll
    for (int v = 0; v < kOut; ++v) o[v] = b4[v];
    for (int k = 0; k < kW; k += 8) {
      const uint4 x = *reinterpret_cast<const uint4*>(H4 + (size_t)r * kW + k);
      const bf16* e = reinterpret_cast<const bf16*>(&x);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float hv = __bfloat162float(e[q]);
#pragma unroll
        for (int v = 0; v < kOut; ++v) o[v] += hv * w[v * kW + k + q];
      }
    }
#pragma unroll
    for (int v = 0; v < kOut; ++v) {
      O[r * 8 + v] = o[v];
      const float d = o[v] - (T ? T[r * kOut + v] : 0.0f);
      if (dO) dO[r * 8 + v] = 2.0f * d / (5.0f * (float)B);
      l += (double)d * (double)d;
    }
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0 && loss_part) loss_part[blockIdx.x] = red[0] / (5.0 * (double)B);
}

// dH4 = dO W4 (fp32 [B][256]) and per-chunk partials of dW4 / db4: part[chunk][5*256 + 5]
__global__ void output_backward_kernel(int B, const float* __restrict__ dO,
                                       const bf16* __restrict__ H4, const float* __restrict__ W4,
                                       float* __restrict__ dH, float* __restrict__ part) {
  const int j = threadIdx.x;  // column
  const int r0 = blockIdx.x * kChunk;
  float w[kOut];
#pragma unroll
  for (int v = 0; v < kOut; ++v) w[v] = W4[v * kW + j];
  float aw[kOut] = {0, 0, 0, 0, 0}, ab[kOut] = {0, 0, 0, 0, 0};
  for (int r = r0; r < r0 + kChunk && r < B; ++r) {
    const float h = __bfloat162float(H4[(size_t)r * kW + j]);
    float s = 0.0f;
#pragma unroll
    for (int v = 0; v < kOut; ++v) {
      const float d = dO[r * 8 + v];
      s += d * w[v];
      aw[v] += d * h;
      ab[v] += d;
    }
    dH[(size_t)r * kW + j] = s;
  }
  float* p = part + (size_t)blockIdx.x * (kOut * kW + kOut);
#pragma unroll
  for (int v = 0; v < kOut; ++v) p[v * kW + j] = aw[v];
  if (j < kOut) p[kOut * kW + j] = ab[j];
}

// FiLM + SiLU backward of one layer: dZ (bf16) for the GEMMs and per-chunk partials
// part[chunk][9][256]: row 0 db, rows 1..3 dF of gamma, rows 4..6 dF of beta, row 7 dg of
// gamma, row 8 dg of beta.
__global__ void film_backward_kernel(int B, const float* __restrict__ dH, const float* __restrict__ Z,
                                     const float* __restrict__ Y, const float* __restrict__ F,
                                     const float* __restrict__ g, const float* __restrict__ C,
                                     bf16* __restrict__ dZ, float* __restrict__ part) {
  const int j = threadIdx.x;
  const int r0 = blockIdx.x * kChunk;
  const float f0 = F[j * 3], f1 = F[j * 3 + 1], f2 = F[j * 3 + 2], gj = g[j];
  float a[8] = {0, 0, 0, 0, 0, 0, 0, 0}, db = 0.0f;
  for (int r = r0; r < r0 + kChunk && r < B; ++r) {
    const float c0 = C[r * 3], c1 = C[r * 3 + 1], c2 = C[r * 3 + 2];
    const float gam = f0 * c0 + f1 * c1 + f2 * c2 + gj;
    const size_t q = (size_t)r * kW + j;
    const float dy = dH[q] * dsilu(Y[q]);
    const float dz = dy * (1.0f + gam);
    const float dgam = dy * Z[q];
    dZ[q] = __float2bfloat16(dz);
    db += dz;
    a[0] += dgam * c0;
    a[1] += dgam * c1;
    a[2] += dgam * c2;
    a[3] += dy * c0;
    a[4] += dy * c1;
    a[5] += dy * c2;
    a[6] += dgam;
    a[7] += dy;
  }
  float* p = part + (size_t)blockIdx.x * 9 * kW;
  p[j] = db;
#pragma unroll
  for (int k = 0; k < 8; ++k) p[(1 + k) * kW + j] = a[k];
}

// out[k] = sum over chunks of part[chunk][k] in chunk order (k < width)
__global__ void reduce_chunks_kernel(int n_chunks, int width, const float* __restrict__ part,
                                     float* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= width) return;
  float s = 0.0f;
  for (int c = 0; c < n_chunks; ++c) s += part[(size_t)c * width + k];
  out[k] = s;
}

// scatter the FiLM partial sums of one layer into the gradient vector
__global__ void film_grad_scatter_kernel(const float* __restrict__ red9, float* __restrict__ gb,
                                         float* __restrict__ gF, float* __restrict__ gg) {
  const int j = threadIdx.x;
  gb[j] = red9[j];
  for (int a = 0; a < 3; ++a) {
    gF[j * 3 + a] = red9[(1 + a) * kW + j];
    gF[(kW + j) * 3 + a] = red9[(4 + a) * kW + j];
  }
  gg[j] = red9[7 * kW + j];
  gg[kW + j] = red9[8 * kW + j];
}

// AdamW on the flat parameters (decoupled weight decay where decay_mask != 0), then the BF16
// copies of the hidden weight matrices
__global__ void adamw_kernel(int64_t n, float* __restrict__ p, const float* __restrict__ grad,
                             float* __restrict__ m, float* __restrict__ v,
                             const uint8_t* __restrict__ decay_mask, float lr, float wd,
                             float bc1, float bc2) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float upd = (mi / bc1) / (sqrtf(vi / bc2) + eps) + (decay_mask[i] ? wd * p[i] : 0.0f);
    p[i] -= lr * upd;
  }
}

__global__ void to_bf16_kernel(int64_t n, const float* __restrict__ x, bf16* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

__global__ void fill_cond_kernel(int B, const float* __restrict__ c3, float* __restrict__ C) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < B)
    for (int a = 0; a < 3; ++a) C[r * 3 + a] = c3[a];
}

}  // namespace

// ---- the handle ------------------------------------------------------------------------------
struct bes_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  std::vector<void*> allocs;
  int64_t nc = 0, n_rows = 0;  // cells, cells rounded up to the row tile
  double gamma = 1.4, R = 287.0;
  Layout L;
  float* feat_xn = nullptr;  // [nc][3] scaled centroids (reference numbering)
  bf16* feat = nullptr;      // [n_rows][64]
  float* p = nullptr;        // parameters, gradient, AdamW moments
  float* grad = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  uint8_t* decay = nullptr;
  bf16* Wb[kLayers] = {};
  int64_t t = 0;             // AdamW steps taken
  double cmean[3] = {0, 0, 0}, csd[3] = {1, 1, 1}, oscale[kOut] = {1, 1, 1, 1, 1};
  // batch buffers (capacity in rows)
  int cap = 0;
  bf16* H[kLayers + 1] = {};
  float* Z[kLayers] = {};
  float* Y[kLayers] = {};
  float *C = nullptr, *T = nullptr, *O = nullptr, *dO = nullptr, *dH = nullptr, *dHk = nullptr;
  bf16* dZ = nullptr;
  float *part = nullptr, *red = nullptr, *wpart = nullptr;
  double* loss_part = nullptr;
  int* gemm_err = nullptr;   // set by a GEMM whose tensor-core wait gave up
  std::vector<bes_mlp*> dummy;
};

namespace {

#define MLP_TRY(h, call)                                                         \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      (h)->last_error = std::string(#call) + ": " + cudaGetErrorString(e_);      \
      return BES_ERR_CUDA;                                                       \
    }                                                                            \
  } while (0)

// BES_ERR_TIMEOUT (and the flag cleared) if a GEMM's wait on the tensor core gave up
int gemm_status(bes_mlp* h) {
  int e = 0;
  MLP_TRY(h, cudaMemcpy(&e, h->gemm_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (!e) return BES_OK;
  cudaMemset(h->gemm_err, 0, sizeof(int));
  h->last_error = "a tensor-core GEMM stopped waiting for its products after two seconds";
  return BES_ERR_TIMEOUT;
}

template <class X>
int mlp_alloc(bes_mlp* h, X** ptr, size_t count) {
  *ptr = nullptr;
  cudaError_t e = cudaMalloc((void**)ptr, std::max<size_t>(count, 1) * sizeof(X));
  if (e != cudaSuccess) {
    h->last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return BES_ERR_CUDA;
  }
  h->allocs.push_back(*ptr);
  return BES_OK;
}

int ensure_batch(bes_mlp* h, int B) {
  if (B <= h->cap) return BES_OK;
  int rc = 0;
  for (int l = 0; l <= kLayers; ++l) rc |= mlp_alloc(h, &h->H[l], (size_t)B * (l == 0 ? kK0 : kW));
  for (int l = 0; l < kLayers; ++l) {
    rc |= mlp_alloc(h, &h->Z[l], (size_t)B * kW);
    rc |= mlp_alloc(h, &h->Y[l], (size_t)B * kW);
  }
  rc |= mlp_alloc(h, &h->C, (size_t)B * 3);
  rc |= mlp_alloc(h, &h->T, (size_t)B * kOut);
  rc |= mlp_alloc(h, &h->O, (size_t)B * 8);
  rc |= mlp_alloc(h, &h->dO, (size_t)B * 8);
  rc |= mlp_alloc(h, &h->dH, (size_t)B * kW);
  rc |= mlp_alloc(h, &h->dHk, (size_t)B * kW);
  rc |= mlp_alloc(h, &h->dZ, (size_t)B * kW);
  const int chunks = (B + kChunk - 1) / kChunk;
  rc |= mlp_alloc(h, &h->part, (size_t)chunks * std::max(9 * kW, kOut * kW + kOut));
  rc |= mlp_alloc(h, &h->red, (size_t)9 * kW);
  // split-K partials of dW: B / 512 splits of [256][256]
  rc |= mlp_alloc(h, &h->wpart, (size_t)std::max(1, B / 512) * kW * kW);
  rc |= mlp_alloc(h, &h->loss_part, (size_t)(B + 255) / 256);
  if (rc) return BES_ERR_CUDA;
  h->cap = B;
  return BES_OK;
}

inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

// C = A(m,k) B(k,n) with optional split over k (partials at C + z*M*ldc)
template <bool A_T, bool B_T>
void gemm(cudaStream_t s, int M, int N, int K, const bf16* A, int lda, const bf16* B, int ldb,
          float* C, int ldc, int splits, int* err) {
  dim3 grid(N / GBN, M / GBM, splits);
  gemm_tc_kernel<A_T, B_T><<<grid, 128, 0, s>>>(M, N, A, lda, B, ldb, C, ldc, K / splits, err);
}

// forward of B rows whose features are in h->H[0] and conditions in h->C; outputs in h->O
void forward(bes_mlp* h, int B) {
  cudaStream_t s = h->stream;
  const int fb = std::min(B, 4096);
  for (int l = 0; l < kLayers; ++l) {
    const int k = l == 0 ? kK0 : kW;
    gemm<false, false>(s, B, kW, k, h->H[l], k, h->Wb[l], k, h->Z[l], kW, 1, h->gemm_err);
    film_forward_kernel<<<fb, kW, 0, s>>>(B, h->Z[l], h->p + h->L.b[l], h->p + h->L.F[l],
                                          h->p + h->L.g[l], h->C, h->Y[l], h->H[l + 1]);
  }
}

// loss, gradient of the batch in h->H[0], h->C, h->T into h->grad; loss partials in loss_part
void backward(bes_mlp* h, int B) {
  cudaStream_t s = h->stream;
  const Layout& L = h->L;
  const int chunks = nblk(B, kChunk);
  output_forward_kernel<<<nblk(B, 256), 256, 0, s>>>(B, h->H[kLayers], h->p + L.W[4], h->p + L.b[4],
                                                      h->T, h->O, h->dO, h->loss_part);
  output_backward_kernel<<<chunks, kW, 0, s>>>(B, h->dO, h->H[kLayers], h->p + L.W[4], h->dH,
                                               h->part);
  reduce_chunks_kernel<<<nblk(kOut * kW + kOut, 256), 256, 0, s>>>(chunks, kOut * kW + kOut, h->part,
                                                                   h->grad + L.W[4]);
  float* dHin = h->dH;
  for (int l = kLayers - 1; l >= 0; --l) {
    const int k = l == 0 ? kK0 : kW;
    film_backward_kernel<<<chunks, kW, 0, s>>>(B, dHin, h->Z[l], h->Y[l], h->p + L.F[l],
                                               h->p + L.g[l], h->C, h->dZ, h->part);
    reduce_chunks_kernel<<<nblk(9 * kW, 256), 256, 0, s>>>(chunks, 9 * kW, h->part, h->red);
    film_grad_scatter_kernel<<<1, kW, 0, s>>>(h->red, h->grad + L.b[l], h->grad + L.F[l],
                                              h->grad + L.g[l]);
    // dW_l = dZ^T H_l, split over the rows in chunks of 512 when they divide the batch
    const int splits = B % 512 == 0 ? B / 512 : 1;
    gemm<true, true>(s, kW, k, B, h->dZ, kW, h->H[l], k, h->wpart, k, splits, h->gemm_err);
    reduce_chunks_kernel<<<nblk((int64_t)kW * k, 256), 256, 0, s>>>(splits, kW * k, h->wpart,
                                                                    h->grad + L.W[l]);
    if (l > 0) {
      // dH_l = dZ W_l (W_l is [256][256], element (k, n) at k*256 + n)
      float* dHout = dHin == h->dH ? h->dHk : h->dH;
      gemm<false, true>(s, B, kW, kW, h->dZ, kW, h->Wb[l], kW, dHout, kW, 1, h->gemm_err);
      dHin = dHout;
    }
  }
}

void adamw(bes_mlp* h, double lr, double wd) {
  h->t += 1;
  const float bc1 = (float)(1.0 - std::pow(0.9, (double)h->t));
  const float bc2 = (float)(1.0 - std::pow(0.999, (double)h->t));
  adamw_kernel<<<1024, 256, 0, h->stream>>>(h->L.n, h->p, h->grad, h->m, h->v, h->decay, (float)lr,
                                            (float)wd, bc1, bc2);
  for (int l = 0; l < kLayers; ++l) {
    const int64_t n = (int64_t)kW * (l == 0 ? kK0 : kW);
    to_bf16_kernel<<<256, 256, 0, h->stream>>>(n, h->p + h->L.W[l], h->Wb[l]);
  }
}

void freestream_conserved(double gamma, double R, const double* mach, double* U) {
  // rho = 1, p = 1/gamma, T = 1/(gamma R) (Config.cpp:480-488), cv = R/(gamma-1)
  const double cv = R / (gamma - 1.0), T = 1.0 / (gamma * R);
  double q = 0.0;
  for (int d = 0; d < 3; ++d) q += mach[d] * mach[d];
  U[0] = 1.0;
  for (int d = 0; d < 3; ++d) U[1 + d] = mach[d];
  U[4] = cv * T + q / 2.0;
}

int check_rows(bes_mlp* h, int64_t B) {
  if (B < kRowTile || B % kRowTile != 0 || B > (1 << 22)) {
    h->last_error = "batch must be a positive multiple of 128 rows and at most 4,194,304";
    return BES_ERR_INVALID;
  }
  return BES_OK;
}

}  // namespace

extern "C" {

int bes_mlp_create(const bes_ctx* ctx, uint64_t seed, bes_mlp** out) {
  if (!ctx || !out) return BES_ERR_INVALID;
  *out = nullptr;
  bes_mlp* h = new bes_mlp();
  h->device = ctx->device;
  cudaSetDevice(h->device);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return BES_ERR_CUDA;
  }
  h->gamma = ctx->opt.specific_heat_ratio;
  h->R = ctx->opt.gas_constant;
  h->nc = ctx->ref.nc;
  h->n_rows = (h->nc + kRowTile - 1) / kRowTile * kRowTile;
  // centroids scaled by their bounding box (reference numbering)
  std::vector<float> xn((size_t)h->nc * 3);
  for (int a = 0; a < 3; ++a) {
    double lo = 1e300, hi = -1e300;
    for (int64_t i = 0; i < h->nc; ++i) {
      lo = std::min(lo, ctx->ref.centroid[i * 3 + a]);
      hi = std::max(hi, ctx->ref.centroid[i * 3 + a]);
    }
    const double span = hi > lo ? hi - lo : 1.0;
    for (int64_t i = 0; i < h->nc; ++i)
      xn[i * 3 + a] = (float)(2.0 * (ctx->ref.centroid[i * 3 + a] - lo) / span - 1.0);
  }
  const Layout& L = h->L;
  int rc = 0;
  rc |= mlp_alloc(h, &h->feat_xn, xn.size());
  rc |= mlp_alloc(h, &h->feat, (size_t)h->n_rows * kK0);
  rc |= mlp_alloc(h, &h->p, L.n);
  rc |= mlp_alloc(h, &h->grad, L.n);
  rc |= mlp_alloc(h, &h->m, L.n);
  rc |= mlp_alloc(h, &h->v, L.n);
  rc |= mlp_alloc(h, &h->decay, L.n);
  for (int l = 0; l < kLayers; ++l) rc |= mlp_alloc(h, &h->Wb[l], (size_t)kW * (l == 0 ? kK0 : kW));
  rc |= mlp_alloc(h, &h->gemm_err, 1);
  if (rc) {
    bes_mlp_destroy(h);
    return BES_ERR_CUDA;
  }
  cudaMemset(h->gemm_err, 0, sizeof(int));
  // Glorot-uniform weights from the seed, zero biases, identity FiLM (F = 0, g = 0), a small
  // output layer
  std::vector<float> p(L.n, 0.0f);
  std::vector<uint8_t> decay(L.n, 0);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 12345;
  auto uni = [&]() { st = mix64(st); return (double)(st >> 11) * (1.0 / 9007199254740992.0); };
  for (int l = 0; l <= kLayers; ++l) {
    const int fin = l == 0 ? kK0 : kW, fout = l == kLayers ? kOut : kW;
    const double a = std::sqrt(6.0 / (fin + fout)) * (l == kLayers ? 0.1 : 1.0);
    for (int64_t q = 0; q < (int64_t)fin * fout; ++q) {
      p[L.W[l] + q] = (float)((2.0 * uni() - 1.0) * a);
      decay[L.W[l] + q] = 1;
    }
  }
  cudaMemcpy(h->feat_xn, xn.data(), xn.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(h->p, p.data(), L.n * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(h->decay, decay.data(), L.n, cudaMemcpyHostToDevice);
  cudaMemset(h->m, 0, L.n * sizeof(float));
  cudaMemset(h->v, 0, L.n * sizeof(float));
  cudaMemset(h->grad, 0, L.n * sizeof(float));
  encode_kernel<<<nblk(h->n_rows, 128), 128, 0, h->stream>>>((int)h->nc, (int)h->n_rows,
                                                             h->feat_xn, h->feat);
  for (int l = 0; l < kLayers; ++l) {
    const int64_t n = (int64_t)kW * (l == 0 ? kK0 : kW);
    to_bf16_kernel<<<256, 256, 0, h->stream>>>(n, h->p + L.W[l], h->Wb[l]);
  }
  if (cudaStreamSynchronize(h->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    bes_mlp_destroy(h);
    return BES_ERR_CUDA;
  }
  *out = h;
  return BES_OK;
}

void bes_mlp_destroy(bes_mlp* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void* q : h->allocs) cudaFree(q);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

const char* bes_mlp_last_error(const bes_mlp* h) { return h ? h->last_error.c_str() : "null"; }

int bes_mlp_params(bes_mlp* h, float* get, const float* set, int64_t* n_params) {
  if (!h) return BES_ERR_INVALID;
  if (n_params) *n_params = h->L.n;
  if (set) {
    MLP_TRY(h, cudaMemcpy(h->p, set, h->L.n * sizeof(float), cudaMemcpyHostToDevice));
    for (int l = 0; l < kLayers; ++l) {
      const int64_t n = (int64_t)kW * (l == 0 ? kK0 : kW);
      to_bf16_kernel<<<256, 256, 0, h->stream>>>(n, h->p + h->L.W[l], h->Wb[l]);
    }
    MLP_TRY(h, cudaStreamSynchronize(h->stream));
  }
  if (get) MLP_TRY(h, cudaMemcpy(get, h->p, h->L.n * sizeof(float), cudaMemcpyDeviceToHost));
  return BES_OK;
}

int bes_mlp_features(bes_mlp* h, float* xn) {
  if (!h || !xn) return BES_ERR_INVALID;
  MLP_TRY(h, cudaMemcpy(xn, h->feat_xn, h->nc * 3 * sizeof(float), cudaMemcpyDeviceToHost));
  return BES_OK;
}

int bes_mlp_loss_grad(bes_mlp* h, int32_t n_rows, const int64_t* cells, const double* cond,
                      const double* targets, double* loss, float* grad, double* outputs) {
  if (!h || !cells || !cond) return BES_ERR_INVALID;
  int rc = check_rows(h, n_rows);
  if (rc) return rc;
  if ((rc = ensure_batch(h, n_rows))) return rc;
  const int B = n_rows;
  // rows from the feature table, conditions and targets as given
  std::vector<float> C((size_t)B * 3), T((size_t)B * kOut, 0.0f);
  for (int r = 0; r < B; ++r) {
    if (cells[r] < 0 || cells[r] >= h->nc) {
      h->last_error = "cell index out of range";
      return BES_ERR_INVALID;
    }
    for (int a = 0; a < 3; ++a) C[r * 3 + a] = (float)cond[r * 3 + a];
    if (targets)
      for (int v = 0; v < kOut; ++v) T[r * kOut + v] = (float)targets[r * kOut + v];
  }
  for (int r = 0; r < B; ++r)
    MLP_TRY(h, cudaMemcpyAsync(h->H[0] + (size_t)r * kK0, h->feat + (size_t)cells[r] * kK0,
                               kK0 * sizeof(bf16), cudaMemcpyDeviceToDevice, h->stream));
  MLP_TRY(h, cudaMemcpyAsync(h->C, C.data(), C.size() * 4, cudaMemcpyHostToDevice, h->stream));
  MLP_TRY(h, cudaMemcpyAsync(h->T, T.data(), T.size() * 4, cudaMemcpyHostToDevice, h->stream));
  forward(h, B);
  backward(h, B);
  std::vector<double> lp((B + 255) / 256);
  MLP_TRY(h, cudaMemcpyAsync(lp.data(), h->loss_part, lp.size() * 8, cudaMemcpyDeviceToHost, h->stream));
  std::vector<float> o((size_t)B * 8);
  MLP_TRY(h, cudaMemcpyAsync(o.data(), h->O, o.size() * 4, cudaMemcpyDeviceToHost, h->stream));
  if (grad) MLP_TRY(h, cudaMemcpyAsync(grad, h->grad, h->L.n * 4, cudaMemcpyDeviceToHost, h->stream));
  MLP_TRY(h, cudaStreamSynchronize(h->stream));
  MLP_TRY(h, cudaGetLastError());
  if (loss) {
    double s = 0.0;
    for (double x : lp) s += x;
    *loss = s;
  }
  if (outputs)
    for (int r = 0; r < B; ++r)
      for (int v = 0; v < kOut; ++v) outputs[r * kOut + v] = o[r * 8 + v];
  return gemm_status(h);
}

int bes_mlp_apply_grad(bes_mlp* h, const float* grad, double lr, double weight_decay) {
  if (!h || !grad) return BES_ERR_INVALID;
  MLP_TRY(h, cudaMemcpyAsync(h->grad, grad, h->L.n * 4, cudaMemcpyHostToDevice, h->stream));
  adamw(h, lr, weight_decay);
  MLP_TRY(h, cudaStreamSynchronize(h->stream));
  MLP_TRY(h, cudaGetLastError());
  return BES_OK;
}

int bes_mlp_train(bes_mlp* h, int32_t n_samples, const double* mach, const double* U,
                  int64_t steps, int32_t batch, double lr, double weight_decay, uint64_t seed,
                  double* loss_history) {
  if (!h || !mach || !U || n_samples < 1 || steps < 0) return BES_ERR_INVALID;
  int rc = check_rows(h, batch);
  if (rc) return rc;
  if ((rc = ensure_batch(h, batch))) return rc;
  const int64_t nc = h->nc;
  // normalisation from the training set: condition mean / std, output scale = std of U - U_inf
  for (int a = 0; a < 3; ++a) {
    double s = 0, s2 = 0;
    for (int q = 0; q < n_samples; ++q) s += mach[q * 3 + a];
    const double mu = s / n_samples;
    for (int q = 0; q < n_samples; ++q) s2 += (mach[q * 3 + a] - mu) * (mach[q * 3 + a] - mu);
    const double sd = std::sqrt(s2 / n_samples);
    h->cmean[a] = mu;
    h->csd[a] = sd > 1e-6 ? sd : 1.0;
  }
  std::vector<double> Uinf((size_t)n_samples * kOut);
  for (int q = 0; q < n_samples; ++q) freestream_conserved(h->gamma, h->R, &mach[q * 3], &Uinf[q * kOut]);
  for (int v = 0; v < kOut; ++v) {
    double s2 = 0.0;
    for (int q = 0; q < n_samples; ++q)
      for (int64_t i = 0; i < nc; ++i) {
        const double d = U[((size_t)q * nc + i) * kOut + v] - Uinf[q * kOut + v];
        s2 += d * d;
      }
    const double sd = std::sqrt(s2 / ((double)n_samples * nc));
    h->oscale[v] = sd > 1e-6 ? sd : 1e-6;
  }
  std::vector<float> tgt((size_t)n_samples * nc * kOut), cnd((size_t)n_samples * 3);
  for (int q = 0; q < n_samples; ++q) {
    for (int a = 0; a < 3; ++a) cnd[q * 3 + a] = (float)((mach[q * 3 + a] - h->cmean[a]) / h->csd[a]);
    for (int64_t i = 0; i < nc; ++i)
      for (int v = 0; v < kOut; ++v) {
        const size_t k = ((size_t)q * nc + i) * kOut + v;
        tgt[k] = (float)((U[k] - Uinf[q * kOut + v]) / h->oscale[v]);
      }
  }
  float *dt = nullptr, *dc = nullptr;
  MLP_TRY(h, cudaMalloc((void**)&dt, tgt.size() * sizeof(float)));
  if (cudaMalloc((void**)&dc, cnd.size() * sizeof(float)) != cudaSuccess) {
    cudaFree(dt);
    h->last_error = "cudaMalloc of the condition table failed";
    return BES_ERR_CUDA;
  }
  cudaMemcpyAsync(dt, tgt.data(), tgt.size() * 4, cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(dc, cnd.data(), cnd.size() * 4, cudaMemcpyHostToDevice, h->stream);
  std::vector<double> lp((batch + 255) / 256);
  double* dloss = nullptr;
  if (loss_history && steps > 0) cudaMalloc((void**)&dloss, steps * lp.size() * sizeof(double));
  for (int64_t s = 0; s < steps; ++s) {
    gather_kernel<<<nblk(batch, 128), 128, 0, h->stream>>>(batch, seed, s, n_samples, (int)nc,
                                                           h->feat, dt, dc, h->H[0], h->C, h->T);
    forward(h, batch);
    backward(h, batch);
    if (dloss)
      cudaMemcpyAsync(dloss + s * lp.size(), h->loss_part, lp.size() * 8,
                      cudaMemcpyDeviceToDevice, h->stream);
    adamw(h, lr, weight_decay);
  }
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess && dloss) {
    std::vector<double> all(steps * lp.size());
    e = cudaMemcpy(all.data(), dloss, all.size() * 8, cudaMemcpyDeviceToHost);
    for (int64_t s = 0; s < steps; ++s) {
      double x = 0.0;
      for (size_t q = 0; q < lp.size(); ++q) x += all[s * lp.size() + q];
      loss_history[s] = x;
    }
  }
  cudaFree(dt);
  cudaFree(dc);
  if (dloss) cudaFree(dloss);
  if (e != cudaSuccess) {
    h->last_error = std::string("training: ") + cudaGetErrorString(e);
    return BES_ERR_CUDA;
  }
  return gemm_status(h);
}

int bes_mlp_infer(bes_mlp* h, int32_t n, const double* mach, double* U) {
  if (!h || !mach || !U || n < 0) return BES_ERR_INVALID;
  const int B = (int)std::min<int64_t>(h->n_rows, 65536);
  int rc = ensure_batch(h, B);
  if (rc) return rc;
  std::vector<float> o((size_t)B * 8);
  float* dc3 = h->T;  // 3 floats of scratch for the condition
  for (int q = 0; q < n; ++q) {
    float c3[3];
    for (int a = 0; a < 3; ++a) c3[a] = (float)((mach[q * 3 + a] - h->cmean[a]) / h->csd[a]);
    double Uinf[kOut];
    freestream_conserved(h->gamma, h->R, &mach[q * 3], Uinf);
    MLP_TRY(h, cudaMemcpyAsync(dc3, c3, sizeof(c3), cudaMemcpyHostToDevice, h->stream));
    fill_cond_kernel<<<nblk(B, 256), 256, 0, h->stream>>>(B, dc3, h->C);
    for (int64_t r0 = 0; r0 < h->n_rows; r0 += B) {
      const int nb = (int)std::min<int64_t>(B, h->n_rows - r0);
      MLP_TRY(h, cudaMemcpyAsync(h->H[0], h->feat + (size_t)r0 * kK0, (size_t)nb * kK0 * sizeof(bf16),
                                 cudaMemcpyDeviceToDevice, h->stream));
      forward(h, nb);
      output_forward_kernel<<<nblk(nb, 256), 256, 0, h->stream>>>(
          nb, h->H[kLayers], h->p + h->L.W[4], h->p + h->L.b[4], nullptr, h->O, nullptr, nullptr);
      MLP_TRY(h, cudaMemcpyAsync(o.data(), h->O, (size_t)nb * 8 * 4, cudaMemcpyDeviceToHost, h->stream));
      MLP_TRY(h, cudaStreamSynchronize(h->stream));
      for (int r = 0; r < nb && r0 + r < h->nc; ++r)
        for (int v = 0; v < kOut; ++v)
          U[((size_t)q * h->nc + r0 + r) * kOut + v] = Uinf[v] + h->oscale[v] * o[r * 8 + v];
    }
  }
  MLP_TRY(h, cudaGetLastError());
  return gemm_status(h);
}

int bes_mlp_init_state(bes_mlp* h, bes_ctx* ctx, int32_t* used) {
  if (!h || !ctx) return BES_ERR_INVALID;
  if (ctx->ref.nc != h->nc) {
    h->last_error = "the context's mesh differs from the network's";
    return BES_ERR_INVALID;
  }
  const int nb = ctx->nb;
  const int64_t nc = h->nc;
  std::vector<double> mach((size_t)nb * 3);
  for (int b = 0; b < nb; ++b)
    for (int d = 0; d < 3; ++d) mach[b * 3 + d] = ctx->pinf0_host[6 * b + 1 + d];
  std::vector<double> U((size_t)nb * nc * kOut);
  int rc = bes_mlp_infer(h, nb, mach.data(), U.data());
  if (rc) return rc;
  // a prediction that is not physical falls back to the freestream for that condition
  std::vector<double> Uf((size_t)nb * nc * kOut);
  rc = bes_set_freestream_state(ctx);
  if (rc) return rc;
  rc = bes_get_state(ctx, Uf.data());
  if (rc) return rc;
  const double gm1 = h->gamma - 1.0;
  for (int b = 0; b < nb; ++b) {
    bool ok = true;
    for (int64_t i = 0; i < nc && ok; ++i) {
      const double* u = &U[((size_t)b * nc + i) * kOut];
      const double p = gm1 * (u[4] - (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / (2.0 * u[0]));
      ok = u[0] > 0.0 && p > 0.0 && std::isfinite(p);
    }
    if (used) used[b] = ok ? 1 : 0;
    if (!ok)
      std::copy(Uf.begin() + (size_t)b * nc * kOut, Uf.begin() + (size_t)(b + 1) * nc * kOut,
                U.begin() + (size_t)b * nc * kOut);
  }
  return bes_set_state(ctx, U.data());
}

int bes_mlp_normalisation(const bes_mlp* h, double* out) {
  if (!h || !out) return BES_ERR_INVALID;
  for (int a = 0; a < 3; ++a) {
    out[a] = h->cmean[a];
    out[3 + a] = h->csd[a];
  }
  for (int v = 0; v < kOut; ++v) out[6 + v] = h->oscale[v];
  return BES_OK;
}

}  // extern "C"
