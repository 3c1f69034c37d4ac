// Krylov side of the implicit path, batched over conditions ("slots"): preconditioner sweeps,
// matrix-vector products, Gram-Schmidt, and the GMRES control (Givens rotations, least
// squares, restart and convergence decisions) on the device, so that a whole linear solve
// runs inside one CUDA graph with conditional nodes and the host is not asked between
// Arnoldi steps.
//
// Slots: every kernel takes its slot from blockIdx.y.  A per-slot array is a SlotPtr: the
// first slot's address and the stride to the next slot (0 for an array all slots share).  A
// kernel given a run-flag array returns at once for a slot whose flag is 0 (a converged or
// frozen condition), so finished slots cost no memory traffic.
//
// The Krylov-side vectors (right-hand side b, iterates, basis, preconditioner output) are
// cell-major: component v of cell i is x[i*5 + v], so a neighbour's five values are one
// 20-byte gather.
#pragma once
#include <cuda_fp16.h>

#include <type_traits>

#include "implicit_kernels.cuh"

namespace bes {

template <class T>
struct SlotPtr {
  T* p;
  int64_t stride;
  __device__ __forceinline__ T* at() const { return p + (int64_t)blockIdx.y * stride; }
  __device__ __forceinline__ T* of(int k) const { return p + (int64_t)k * stride; }
};
template <class T>
inline SlotPtr<T> slots(T* p, int64_t stride) { return SlotPtr<T>{p, stride}; }
template <class T>
inline SlotPtr<const T> cslots(const T* p, int64_t stride) { return SlotPtr<const T>{p, stride}; }

// The slot's array: with BATCH false (a single-condition context) the first slot's pointer
// itself, so that the hot gather kernels keep their pointers in the parameter bank instead of
// computing per-slot addresses into registers.
template <bool BATCH, class T>
__device__ __forceinline__ T* sat(const SlotPtr<T>& s) {
  if constexpr (BATCH) return s.at();
  else return s.p;
}

__device__ __forceinline__ bool slot_idle(const int32_t* run) {
  return run != nullptr && run[blockIdx.y] == 0;
}

// ---- matrix words read once per application --------------------------------------------------
// The packed matrix and factor words are read once per SpMV or preconditioner application, and
// their stream is several times larger than L2.  Under the default policy it evicts the Krylov
// vectors whose values the neighbour gathers read again, and every gathered neighbour costs a
// DRAM sector: the 2.16M-cell SpMV read 829 MB from DRAM against 696 MB of compulsory traffic.
// Loaded with an evict_first policy the matrix words leave the vectors in L2 (696 MB).
// ld_once is a read-only (non-coherent) load that the compiler may move: only for words that
// no thread writes while the kernel runs.
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ __half2 ld_once(const __half2* a, uint64_t pol) {
  uint32_t v;
  asm("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
  return *reinterpret_cast<const __half2*>(&v);
}
__device__ __forceinline__ float ld_once(const float* a, uint64_t pol) {
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ uint4 ld_once(const uint4* a, uint64_t pol) {
  uint4 v;
  asm("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
      : "l"(a), "l"(pol));
  return v;
}
// load_packed with the evict_first policy
__device__ __forceinline__ void load_packed_once(const __half2* __restrict__ H, int s, int nc, int i,
                                                 float* a, uint64_t pol) {
#pragma unroll
  for (int p = 0; p < 13; ++p) {
    const float2 f = __half22float2(ld_once(H + (int64_t)(s * 13 + p) * nc + i, pol));
    a[2 * p] = f.x;
    a[2 * p + 1] = f.y;
  }
}

// ---- gathers of a cell's five values ------------------------------------------------------------
// A Krylov vector holds a cell's five FP32 values in 20 consecutive bytes, which always lie in
// two aligned 16-byte chunks.  Loading those two chunks takes two load instructions per
// neighbour instead of five (for a warp whose neighbours are scattered, one L1 wavefront per
// lane and instruction).  The vectors are 16-byte aligned and have at least 16 bytes after the
// last cell of every slot (the vector stride), so both chunks are in bounds.  The values are
// the same floats either way.
__device__ __forceinline__ void gather5(const float* __restrict__ x, int j, float* y) {
  const int64_t e0 = (int64_t)j * 5;
  const float4* p = reinterpret_cast<const float4*>(x) + (e0 >> 2);
  const float4 a = p[0], b = p[1];
  const float w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
  const int o = (int)(e0 & 3);
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    float t = w[v];
    t = o == 1 ? w[v + 1] : t;
    t = o == 2 ? w[v + 2] : t;
    t = o == 3 ? w[v + 3] : t;
    y[v] = t;
  }
}

// ---- preconditioners ------------------------------------------------------------------------

// Load of a Krylov vector entry; COH: through L2 only (ld.global.cg), for values that other
// blocks of the same launch wrote (a persistent sweep: L1 is not coherent across SMs).
template <bool COH, class T>
__device__ __forceinline__ T vld(const T* p) {
  if constexpr (COH) return __ldcg(p);
  else return *p;
}

// Colour-ordered block-ILU(0) sweep when the colours are contiguous cell ranges in increasing
// order (the colour-major numbering): the rows of one colour are [r0, r1), lower neighbours
// are j < r0 and upper neighbours k >= r1, so no row list or position lookup is needed.  The
// lower solve of colour 0 is the identity, so its y values are read from `in` where they are
// needed (lower neighbours in [0, s1), colour 0's own upper solve) instead of being copied.
//   LOWER only        colours 1..C-2 of the forward sweep: out_i = in_i - sum L_ij y_j
//   LOWER and UPPER   the last colour: both solves at once (it has no upper neighbours)
//   UPPER only        colours C-2..0 of the backward sweep: out_i = inv(U_ii)(y_i - sum U_ik z_k)
// `in` and `out` must not alias.
template <class T, bool LOWER, bool UPPER, bool COH = false>
__device__ __forceinline__ void ilu_colour_row(const DevMesh& m, int i, int r0, int r1, int s1,
                                               const T* __restrict__ A,
                                               const T* __restrict__ Dinv,
                                               const T* __restrict__ in, T* __restrict__ out) {
  const int nc = m.nc;
  constexpr bool G = !COH && std::is_same<T, float>::value;  // two-chunk gathers
  const T* own = (LOWER || r0 == 0) ? in : out;
  T acc[5];
  if constexpr (G) {
    gather5(own, i, acc);
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) acc[v] = vld<COH>(own + (int64_t)i * 5 + v);
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int j = m.adj[s * nc + i];
    const bool lower = LOWER && j >= 0 && j < r0;
    const bool upper = UPPER && j >= r1;
    if (!lower && !upper) continue;
    const T* src = (lower && j < s1) ? in : out;
    T y[5];
    if constexpr (G) {
      gather5(src, j, y);
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) y[v] = vld<COH>(src + (int64_t)j * 5 + v);
    }
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] -= ellc(A, 1 + s, r * 5 + c, nc, i) * y[c];
  }
  if (UPPER) {
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      T x = T(0);
#pragma unroll
      for (int c = 0; c < 5; ++c) x += Dinv[(int64_t)(r * 5 + c) * nc + i] * acc[c];
      out[(int64_t)i * 5 + r] = x;
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) out[(int64_t)i * 5 + v] = acc[v];
  }
}

template <class T, bool LOWER, bool UPPER, bool BATCH>
__global__ void __launch_bounds__(128) ilu_colour_kernel(DevMesh m, int r0, int r1, int s1,
                                                         SlotPtr<const T> Ap, SlotPtr<const T> Dp,
                                                         SlotPtr<const T> inp, SlotPtr<T> outp,
                                                         const int32_t* run) {
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1 || slot_idle(run)) return;
  ilu_colour_row<T, LOWER, UPPER>(m, i, r0, r1, s1, sat<BATCH>(Ap), sat<BATCH>(Dp),
                                  sat<BATCH>(inp), sat<BATCH>(outp));
}

template <bool LOWER, bool UPPER, bool COH = false>
__device__ __forceinline__ void ilu_colour_packed_row(
    const DevMesh& m, int i, int r0, int r1, int s1, const __half2* __restrict__ H,
    const float* __restrict__ HS, const __half2* __restrict__ D, const float* __restrict__ DS,
    const float* __restrict__ in, float* __restrict__ out) {
  const int nc = m.nc;
  const uint64_t pol = l2_evict_first();
  const float* own = (LOWER || r0 == 0) ? in : out;
  float acc[5];
  if constexpr (!COH) {
    gather5(own, i, acc);
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) acc[v] = vld<COH>(own + (int64_t)i * 5 + v);
  }
  // the four neighbour ids first (one round trip), then the qualifying slots
  int jn[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) jn[s] = m.adj[s * nc + i];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int j = jn[s];
    const bool lower = LOWER && j >= 0 && j < r0;
    const bool upper = UPPER && j >= r1;
    if (!lower && !upper) continue;
    const float* src = (lower && j < s1) ? in : out;
    const float sc = ld_once(HS + (int64_t)s * nc + i, pol);
    float y[5], a[26];
    if constexpr (!COH) {
      gather5(src, j, y);
#pragma unroll
      for (int v = 0; v < 5; ++v) y[v] *= sc;
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) y[v] = sc * vld<COH>(src + (int64_t)j * 5 + v);
    }
    load_packed_once(H, s, nc, i, a, pol);
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] = fmaf(-a[r * 5 + c], y[c], acc[r]);
  }
  if (UPPER) {
    float a[26];
    load_packed_once(D, 0, nc, i, a, pol);
    const float sc = ld_once(DS + i, pol);
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      float x = 0.0f;
#pragma unroll
      for (int c = 0; c < 5; ++c) x = fmaf(a[r * 5 + c], acc[c], x);
      out[(int64_t)i * 5 + r] = sc * x;
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) out[(int64_t)i * 5 + v] = acc[v];
  }
}

// ilu_colour_kernel with packed factors: L / U blocks in H slots 0..3 (local faces 0..3),
// inv(U_ii) in D (one slot)
template <bool LOWER, bool UPPER, bool BATCH>
__global__ void __launch_bounds__(128) ilu_colour_packed_kernel(
    DevMesh m, int r0, int r1, int s1, SlotPtr<const __half2> Hp, SlotPtr<const float> HSp,
    SlotPtr<const __half2> Dp, SlotPtr<const float> DSp, SlotPtr<const float> inp,
    SlotPtr<float> outp, const int32_t* run) {
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1 || slot_idle(run)) return;
  ilu_colour_packed_row<LOWER, UPPER>(m, i, r0, r1, s1, sat<BATCH>(Hp), sat<BATCH>(HSp),
                                      sat<BATCH>(Dp), sat<BATCH>(DSp), sat<BATCH>(inp),
                                      sat<BATCH>(outp));
}

// The packed colour sweep with every qualifying slot's loads (scale, 16-bit block, the
// neighbour's values) issued before any arithmetic: two dependent round trips per row
// (neighbour ids, then everything else) instead of one per qualifying slot, at the cost of
// registers.  The arithmetic is that of ilu_colour_packed_row in the same order, so the
// results are identical; the autotuner keeps it only where it is faster.
template <bool LOWER, bool UPPER>
__device__ __forceinline__ void ilu_colour_packed_row_ld(
    const DevMesh& m, int i, int r0, int r1, int s1, const __half2* __restrict__ H,
    const float* __restrict__ HS, const __half2* __restrict__ D, const float* __restrict__ DS,
    const float* __restrict__ in, float* __restrict__ out) {
  const int nc = m.nc;
  const uint64_t pol = l2_evict_first();
  const float* own = (LOWER || r0 == 0) ? in : out;
  int jn[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) jn[s] = m.adj[s * nc + i];
  float acc[5];
  gather5(own, i, acc);
  bool q[4];
  __half2 hb[4][13];
  float sc[4], y[4][5];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int j = jn[s];
    const bool lower = LOWER && j >= 0 && j < r0;
    const bool upper = UPPER && j >= r1;
    q[s] = lower || upper;
    if (q[s]) {
      const float* src = (lower && j < s1) ? in : out;
      sc[s] = ld_once(HS + (int64_t)s * nc + i, pol);
#pragma unroll
      for (int p = 0; p < 13; ++p) hb[s][p] = ld_once(H + (int64_t)(s * 13 + p) * nc + i, pol);
      gather5(src, j, y[s]);
    }
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    if (!q[s]) continue;
    float a[26], ys[5];
#pragma unroll
    for (int p = 0; p < 13; ++p) {
      const float2 f = __half22float2(hb[s][p]);
      a[2 * p] = f.x;
      a[2 * p + 1] = f.y;
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) ys[v] = sc[s] * y[s][v];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] = fmaf(-a[r * 5 + c], ys[c], acc[r]);
  }
  if (UPPER) {
    float a[26];
    load_packed_once(D, 0, nc, i, a, pol);
    const float d = ld_once(DS + i, pol);
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      float x = 0.0f;
#pragma unroll
      for (int c = 0; c < 5; ++c) x = fmaf(a[r * 5 + c], acc[c], x);
      out[(int64_t)i * 5 + r] = d * x;
    }
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) out[(int64_t)i * 5 + v] = acc[v];
  }
}

template <bool LOWER, bool UPPER, bool BATCH>
__global__ void __launch_bounds__(128) ilu_colour_packed_ld_kernel(
    DevMesh m, int r0, int r1, int s1, SlotPtr<const __half2> Hp, SlotPtr<const float> HSp,
    SlotPtr<const __half2> Dp, SlotPtr<const float> DSp, SlotPtr<const float> inp,
    SlotPtr<float> outp, const int32_t* run) {
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1 || slot_idle(run)) return;
  ilu_colour_packed_row_ld<LOWER, UPPER>(m, i, r0, r1, s1, sat<BATCH>(Hp), sat<BATCH>(HSp),
                                         sat<BATCH>(Dp), sat<BATCH>(DSp), sat<BATCH>(inp),
                                         sat<BATCH>(outp));
}

// ---- persistent colour sweep ----------------------------------------------------------------
// One launch per preconditioner application: a grid of resident blocks (cooperative launch,
// sized by occupancy) walks the 2C-1 colour stages of the sweep in order, the rows of every
// slot of a stage spread over all its threads, with a grid barrier between stages.  Each row
// computes exactly what the per-colour kernels compute.  Vector values written in one stage
// are read in later stages by other blocks, so those loads go through L2 (vld<true>).
constexpr int kMaxStages = 16;
struct SweepPlan {
  int n;                     // stages
  int s1;                    // end of colour 0
  int r0[kMaxStages], r1[kMaxStages];
  int kind[kMaxStages];      // 0 lower solve, 1 both solves (last colour), 2 upper solve
};

// Grid barrier state (device memory, zero at start): arrivals, generation, error flag.  A
// wait gives up after one second (BES_ERR_TIMEOUT for the host), and once the error flag is
// set every later wait of every launch returns at once, so no launch can hang.
struct GridSync {
  unsigned int* count;
  unsigned int* gen;
  int* error;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// All blocks of the grid arrive before any leaves; false if the wait gave up.
__device__ __forceinline__ bool grid_sync(const GridSync& g) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int good = *(volatile int*)g.error == 0;
    if (good) {
      const unsigned g0 = ld_acquire(g.gen);
      __threadfence();
      const unsigned t = atomicAdd(g.count, 1u);
      if (t == gridDim.x - 1) {
        atomicExch(g.count, 0u);
        __threadfence();
        atomicAdd(g.gen, 1u);
      } else {
        const unsigned long long t0 = global_ns();
        while (ld_acquire(g.gen) == g0) {
          if (*(volatile int*)g.error) {
            good = 0;
            break;
          }
          if (global_ns() - t0 > 1000000000ull) {
            atomicExch(g.error, 1);
            good = 0;
            break;
          }
          __nanosleep(32);
        }
      }
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Operands of a sweep: the factors (packed 16-bit with scales, or T) and the vectors.
template <class T>
struct SweepOps {
  SlotPtr<const __half2> H, D;   // packed: off-diagonal factor blocks, inverse diagonal
  SlotPtr<const float> HS, DS;   // packed: their scales
  SlotPtr<const T> L, Dinv;      // unpacked factors
  SlotPtr<const T> in;
  SlotPtr<T> out;
};

template <class T, bool PACKED>
__global__ void __launch_bounds__(128) ilu_sweep_persistent_kernel(DevMesh m, SweepPlan P,
                                                                   SweepOps<T> O, int nslot,
                                                                   const int32_t* run,
                                                                   GridSync gs) {
  if (*(volatile int*)gs.error) return;
  const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
  for (int st = 0; st < P.n; ++st) {
    const int r0 = P.r0[st], r1 = P.r1[st], kind = P.kind[st];
    const int nrows = r1 - r0;
    const int64_t items = (int64_t)nslot * nrows;
    for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < items; it += nthreads) {
      const int k = (int)(it / nrows);
      const int i = r0 + (int)(it - (int64_t)k * nrows);
      if (run != nullptr && run[k] == 0) continue;
      if constexpr (PACKED) {
        if (kind == 0)
          ilu_colour_packed_row<true, false, true>(m, i, r0, r1, P.s1, O.H.of(k), O.HS.of(k),
                                                   O.D.of(k), O.DS.of(k), O.in.of(k), O.out.of(k));
        else if (kind == 1)
          ilu_colour_packed_row<true, true, true>(m, i, r0, r1, P.s1, O.H.of(k), O.HS.of(k),
                                                  O.D.of(k), O.DS.of(k), O.in.of(k), O.out.of(k));
        else
          ilu_colour_packed_row<false, true, true>(m, i, r0, r1, P.s1, O.H.of(k), O.HS.of(k),
                                                   O.D.of(k), O.DS.of(k), O.in.of(k), O.out.of(k));
      } else {
        if (kind == 0)
          ilu_colour_row<T, true, false, true>(m, i, r0, r1, P.s1, O.L.of(k), O.Dinv.of(k),
                                               O.in.of(k), O.out.of(k));
        else if (kind == 1)
          ilu_colour_row<T, true, true, true>(m, i, r0, r1, P.s1, O.L.of(k), O.Dinv.of(k),
                                              O.in.of(k), O.out.of(k));
        else
          ilu_colour_row<T, false, true, true>(m, i, r0, r1, P.s1, O.L.of(k), O.Dinv.of(k),
                                               O.in.of(k), O.out.of(k));
      }
    }
    if (st + 1 < P.n && !grid_sync(gs)) return;
  }
}

// Level-scheduled block ILU(0) in reverse Cuthill-McKee order: forward solve of one stage,
// out_i = in_i - sum_{lower j} L_ij out_j (in place on out after copy_vec_kernel)
template <class T>
__global__ void __launch_bounds__(128) ilu_lower_kernel(DevMesh m, const int32_t* __restrict__ rows,
                                                        int nrows, const int32_t* __restrict__ pos,
                                                        SlotPtr<const T> Ap, SlotPtr<T> zp,
                                                        const int32_t* run) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows || slot_idle(run)) return;
  const T* __restrict__ A = Ap.at();
  T* z = zp.at();
  const int nc = m.nc;
  const int i = rows[t];
  const int pi = pos[i];
  T acc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = z[(int64_t)i * 5 + v];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int j = m.adj[s * nc + i];
    if (j < 0 || pos[j] >= pi) continue;
    T y[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) y[v] = z[(int64_t)j * 5 + v];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] -= ellc(A, 1 + s, r * 5 + c, nc, i) * y[c];
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) z[(int64_t)i * 5 + v] = acc[v];
}

// backward solve of one stage, in place: z_i = inv(U_ii) (y_i - sum_{upper k} U_ik z_k)
template <class T>
__global__ void __launch_bounds__(128) ilu_upper_kernel(DevMesh m, const int32_t* __restrict__ rows,
                                                        int nrows, const int32_t* __restrict__ pos,
                                                        SlotPtr<const T> Ap, SlotPtr<const T> Dp,
                                                        SlotPtr<T> zp, const int32_t* run) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows || slot_idle(run)) return;
  const T* __restrict__ A = Ap.at();
  const T* __restrict__ Dinv = Dp.at();
  T* z = zp.at();
  const int nc = m.nc;
  const int i = rows[t];
  const int pi = pos[i];
  T acc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = z[(int64_t)i * 5 + v];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int k = m.adj[s * nc + i];
    if (k < 0 || pos[k] <= pi) continue;
    T y[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) y[v] = z[(int64_t)k * 5 + v];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] -= ellc(A, 1 + s, r * 5 + c, nc, i) * y[c];
  }
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    T x = T(0);
#pragma unroll
    for (int c = 0; c < 5; ++c) x += Dinv[(int64_t)(r * 5 + c) * nc + i] * acc[c];
    z[(int64_t)i * 5 + r] = x;
  }
}

// out = in (N elements per slot)
template <class T>
__global__ void __launch_bounds__(256) copy_vec_kernel(SlotPtr<T> outp, SlotPtr<const T> inp,
                                                       int64_t N, const int32_t* run) {
  if (slot_idle(run)) return;
  T* __restrict__ out = outp.at();
  const T* __restrict__ in = inp.at();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x)
    out[idx] = in[idx];
}

// block-Jacobi application: out_i = Dinv_i in_i
template <class T>
__global__ void __launch_bounds__(256) jacobi_apply_kernel(int nc, SlotPtr<const T> Dp,
                                                           SlotPtr<const T> inp, SlotPtr<T> outp,
                                                           const int32_t* run) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc || slot_idle(run)) return;
  const T* __restrict__ Dinv = Dp.at();
  const T* __restrict__ in = inp.at();
  T* __restrict__ out = outp.at();
  T x[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) x[v] = in[(int64_t)i * 5 + v];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    T acc = T(0);
#pragma unroll
    for (int c = 0; c < 5; ++c) acc += Dinv[(int64_t)(r * 5 + c) * nc + i] * x[c];
    out[(int64_t)i * 5 + r] = acc;
  }
}

// block-Jacobi application with a packed inverse diagonal
static __global__ void __launch_bounds__(256) jacobi_apply_packed_kernel(
    int nc, SlotPtr<const __half2> Dp, SlotPtr<const float> DSp, SlotPtr<const float> inp,
    SlotPtr<float> outp, const int32_t* run) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc || slot_idle(run)) return;
  const float* __restrict__ in = inp.at();
  float* __restrict__ out = outp.at();
  float x[5], a[26];
#pragma unroll
  for (int v = 0; v < 5; ++v) x[v] = in[(int64_t)i * 5 + v];
  load_packed(Dp.at(), 0, nc, i, a);
  const float sc = DSp.at()[i];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c < 5; ++c) acc = fmaf(a[r * 5 + c], x[c], acc);
    out[(int64_t)i * 5 + r] = sc * acc;
  }
}

// ---- matrix-vector products ------------------------------------------------------------------

// y = A x (ELL), or y = b - A x when b is given
template <class T, bool BATCH>
__global__ void __launch_bounds__(256) spmv_kernel(DevMesh m, SlotPtr<const T> Ap,
                                                   SlotPtr<const T> xp, SlotPtr<const T> bp,
                                                   SlotPtr<T> yp, const int32_t* run) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = m.nc;
  if (i >= nc || slot_idle(run)) return;
  const T* __restrict__ A = sat<BATCH>(Ap);
  const T* __restrict__ x = sat<BATCH>(xp);
  const T* __restrict__ b = bp.p ? sat<BATCH>(bp) : nullptr;
  T* __restrict__ y = sat<BATCH>(yp);
  constexpr bool G = std::is_same<T, float>::value;  // two-chunk gathers
  T acc[5], xi[5];
  if constexpr (G) {
    gather5(x, i, xi);
  } else {
#pragma unroll
    for (int v = 0; v < 5; ++v) xi[v] = x[(int64_t)i * 5 + v];
  }
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    T s = T(0);
#pragma unroll
    for (int c = 0; c < 5; ++c) s += ellc(A, 0, r * 5 + c, nc, i) * xi[c];
    acc[r] = s;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j = m.adj[q * nc + i];
    if (j < 0) continue;
    if constexpr (G) {
      gather5(x, j, xi);
    } else {
#pragma unroll
      for (int v = 0; v < 5; ++v) xi[v] = x[(int64_t)j * 5 + v];
    }
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] += ellc(A, 1 + q, r * 5 + c, nc, i) * xi[c];
  }
#pragma unroll
  for (int r = 0; r < 5; ++r)
    y[(int64_t)i * 5 + r] = b ? b[(int64_t)i * 5 + r] - acc[r] : acc[r];
}

// y = A x (or b - A x) with A in packed form: per block, the neighbour's values are scaled
// by the block's scale and multiplied by the 16-bit entries
template <bool BATCH>
__global__ void __launch_bounds__(256) spmv_packed_kernel(
    DevMesh m, SlotPtr<const __half2> Hp, SlotPtr<const float> Sp, SlotPtr<const float> xp,
    SlotPtr<const float> bp, SlotPtr<float> yp, const int32_t* run) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = m.nc;
  if (i >= nc || slot_idle(run)) return;
  const __half2* __restrict__ H = sat<BATCH>(Hp);
  const float* __restrict__ S = sat<BATCH>(Sp);
  const float* __restrict__ x = sat<BATCH>(xp);
  const float* __restrict__ b = bp.p ? sat<BATCH>(bp) : nullptr;
  float* __restrict__ y = sat<BATCH>(yp);
  float acc[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  // branch-free, so that every slot's loads can be in flight together: the block of a slot
  // without a neighbour is zero (boundary face, or the empty fourth slot of a triangle), and
  // the row's own values stand in for the missing neighbour's, adding exactly 0
  int jn[5];
  jn[0] = i;
#pragma unroll
  for (int s = 1; s < 5; ++s) {
    const int j = m.adj[(s - 1) * nc + i];
    jn[s] = j >= 0 ? j : i;
  }
  const uint64_t pol = l2_evict_first();
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const float sc = ld_once(S + (int64_t)s * nc + i, pol);
    float xs[5], a[26];
    gather5(x, jn[s], xs);
#pragma unroll
    for (int v = 0; v < 5; ++v) xs[v] *= sc;
    load_packed_once(H, s, nc, i, a, pol);
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] = fmaf(a[r * 5 + c], xs[c], acc[r]);
  }
#pragma unroll
  for (int r = 0; r < 5; ++r)
    y[(int64_t)i * 5 + r] = b ? b[(int64_t)i * 5 + r] - acc[r] : acc[r];
}

// ---- reductions ------------------------------------------------------------------------------

// Per-thread accumulation type of the vector kernels: the FP32 system accumulates each
// thread's few elements in FP32 (the FP64 pipe is ~60x slower on this GPU) and reduces
// across threads and blocks in FP64; the FP64 system stays FP64 throughout.
template <class T> struct AccType { typedef double type; };
template <> struct AccType<float> { typedef float type; };

// Warp sum in the accumulation type.
template <class A>
__device__ __forceinline__ A warp_sum_t(A x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Block reduction of NV per-thread accumulators; partials[k*gridDim.x + blk] (FP64).  Lanes
// are summed in the accumulation type; each warp's sum is widened to FP64 once and the block's
// eight warp sums are added in FP64 in a fixed order.
template <int NV, class A>
__device__ __forceinline__ void block_reduce_store(A (&acc)[NV], double* partials) {
  __shared__ double sh[NV][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const A s = warp_sum_t<A>(acc[k]);
    if (lane == 0) sh[k][wid] = (double)s;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < NV; k += blockDim.x) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += sh[k][q];
    partials[(int64_t)k * gridDim.x + blockIdx.x] = s;
  }
}

// Reduce rows of per-block partials in a fixed order (one block per row, blockIdx.x; slot
// blockIdx.y): out[row] = sum, sqrt(sum) when sqrt_sums, or max for rows >= nsum.
static __global__ void __launch_bounds__(256) reduce_slots_kernel(
    SlotPtr<const double> pp, int nblocks, int nsum, int sqrt_sums, SlotPtr<double> outp,
    const int32_t* run) {
  if (slot_idle(run)) return;
  const double* __restrict__ partials = pp.at();
  __shared__ double sh[8];
  const int k = blockIdx.x;
  const bool is_sum = k < nsum;
  double x = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    const double y = partials[(int64_t)k * nblocks + b];
    x = is_sum ? x + y : fmax(x, y);
  }
  x = is_sum ? warp_sum(x) : warp_max(x);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = x;
  __syncthreads();
  if (threadIdx.x < 32) {
    x = lane < 8 ? sh[lane] : 0.0;
    x = is_sum ? warp_sum(x) : warp_max(x);
    if (lane == 0) outp.at()[k] = (is_sum && sqrt_sums) ? sqrt(x) : x;
  }
}

// ---- Gram-Schmidt of the Arnoldi step -------------------------------------------------
// Classical Gram-Schmidt with a conditional second pass (the oracle's linsolve.hpp gmres
// states the same algorithm):
//   pass 1   h = V^T w and |w|^2 in one read of V and w (gs_dots_kernel);
//   decide   |w - V h|^2 = |w|^2 - |h|^2 (Pythagoras); a second pass runs only when this
//            is <= kReorthTheta2 |w|^2 (gs_decide_kernel, on the device);
//   no second pass: V_{j+1} = (w - V h) / sqrt(|w|^2 - |h|^2) in one more read of V and w
//            (gs_update_kernel<FINAL1>);
//   second pass: w -= V h with V^T w and |w|^2 of the result in the same read
//            (gs_update_kernel<REORTH>), then V_{j+1} = (w - V h2) / norm (<FINAL2>).
// The kernels of the path not taken return at once.  Device scalars per slot (dev):
//   dev[0..nv-1] h, dev[nv] |w|^2; dev[kGsH2 + k] h2, dev[kGsH2 + nv] |w'|^2;
//   dev[kGsFlag] 1 if the second pass runs, dev[kGsInv] 1/h_{j+1,j} (0: leave V_{j+1}),
//   dev[kGsNorm] h_{j+1,j}; dev[kGsR] a vector's squared norm (start and restart).
//   devf: FP32 copies of h, h2, the flag and 1/h_{j+1,j} at the same offsets, written by
//   gs_decide_kernel, so that FP32 update kernels convert nothing per thread.
constexpr double kReorthTheta2 = 1.0 / 16.0;
constexpr int kGsH2 = 40, kGsFlag = 80, kGsInv = 81, kGsNorm = 82, kGsR = 83;
static_assert(kGsR < kGsLd, "Gram-Schmidt scalars per slot");

template <class A>
__device__ __forceinline__ const A* gs_coef(const double* dev, const float* devf);
template <>
__device__ __forceinline__ const double* gs_coef<double>(const double* dev, const float*) {
  return dev;
}
template <>
__device__ __forceinline__ const float* gs_coef<float>(const double*, const float* devf) {
  return devf;
}

// 16-byte unit of the vector kernels; the Krylov vector stride is a multiple of it
template <class T>
struct alignas(16) Pack16 {
  static constexpr int W = 16 / sizeof(T);
  T v[W];
};

// Element type B of the Krylov basis: the vector type T itself, or (precision 2) FP16 holding
// kBasisScale times the value.  A basis vector has unit norm, so |entries| <= 1 and the scaled
// entries stay below 2^14 (FP16 overflows at 65504); entries under 2^-28 lose relative
// precision as FP16 subnormals (absolute error at most 2^-39).
constexpr float kBasisScale = 16384.0f;
constexpr float kBasisInvScale = 1.0f / 16384.0f;

// W consecutive basis entries (16 bytes of basis per access: 16 / sizeof(T) entries of T, or
// eight FP16 entries; W is a multiple of the vector granule Pack16<T>::W)
template <class T, class B>
struct BasisIO {
  static constexpr int W = 16 / sizeof(T);
  template <class A>
  __device__ static __forceinline__ void load(const B* V, int64_t g, A* x) {
    const Pack16<T> p = reinterpret_cast<const Pack16<T>*>(V)[g];
#pragma unroll
    for (int e = 0; e < W; ++e) x[e] = (A)p.v[e];
  }
  // the same with the evict_first policy (a pass over the basis that is not read again soon)
  template <class A>
  __device__ static __forceinline__ void load_once(const B* V, int64_t g, A* x, uint64_t pol) {
    const uint4 u = ld_once(reinterpret_cast<const uint4*>(V) + g, pol);
    const Pack16<T> p = *reinterpret_cast<const Pack16<T>*>(&u);
#pragma unroll
    for (int e = 0; e < W; ++e) x[e] = (A)p.v[e];
  }
  template <class A>
  __device__ static __forceinline__ void store(B* V, int64_t g, const A* x) {
    Pack16<T> p;
#pragma unroll
    for (int e = 0; e < W; ++e) p.v[e] = (T)x[e];
    reinterpret_cast<Pack16<T>*>(V)[g] = p;
  }
  template <class A>
  __device__ static __forceinline__ A get(const B* V, int64_t i) { return (A)V[i]; }
  template <class A>
  __device__ static __forceinline__ void set(B* V, int64_t i, A x) { V[i] = (T)x; }
};
template <>
struct BasisIO<float, __half> {
  static constexpr int W = 8;  // 16-byte loads of eight FP16 entries
  template <class A>
  __device__ static __forceinline__ void load(const __half* V, int64_t g, A* x) {
    unpack(reinterpret_cast<const uint4*>(V)[g], x);
  }
  template <class A>
  __device__ static __forceinline__ void load_once(const __half* V, int64_t g, A* x, uint64_t pol) {
    unpack(ld_once(reinterpret_cast<const uint4*>(V) + g, pol), x);
  }
  template <class A>
  __device__ static __forceinline__ void unpack(const uint4 u, A* x) {
    const unsigned w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&w4[q]));
      x[2 * q] = f.x * kBasisInvScale;
      x[2 * q + 1] = f.y * kBasisInvScale;
    }
  }
  template <class A>
  __device__ static __forceinline__ void store(__half* V, int64_t g, const A* x) {
    unsigned w4[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const __half2 h = __floats2half2_rn(x[2 * q] * kBasisScale, x[2 * q + 1] * kBasisScale);
      w4[q] = *reinterpret_cast<const unsigned*>(&h);
    }
    reinterpret_cast<uint4*>(V)[g] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
  }
  template <class A>
  __device__ static __forceinline__ A get(const __half* V, int64_t i) {
    return __half2float(V[i]) * kBasisInvScale;
  }
  template <class A>
  __device__ static __forceinline__ void set(__half* V, int64_t i, A x) {
    V[i] = __float2half_rn(x * kBasisScale);
  }
};

// Pass 1: partial V_k . w (rows k < NV) and |w|^2 (row NV).
template <class T, class B, int NV>
__global__ void __launch_bounds__(256) gs_dots_kernel(SlotPtr<const B> Vp, int64_t ldv,
                                                      SlotPtr<const T> wp, int64_t N,
                                                      SlotPtr<double> pp, const int32_t* run) {
  if (slot_idle(run)) return;
  typedef typename AccType<T>::type A;
  typedef Pack16<T> P;
  typedef BasisIO<T, B> IO;
  constexpr int W = IO::W;      // entries per granule
  constexpr int NP = W / P::W;  // 16-byte vector packs per granule
  const B* __restrict__ V = Vp.at();
  const T* __restrict__ w = wp.at();
  // the basis with evict_first: w stays in L2 for the update pass that reads it next
  const uint64_t pol = l2_evict_first();
  A acc[NV + 1];
#pragma unroll
  for (int k = 0; k <= NV; ++k) acc[k] = A(0);
  const int64_t ng = N / W;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ng;
       g += (int64_t)gridDim.x * blockDim.x) {
    A wv[W];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const P q = reinterpret_cast<const P*>(w)[g * NP + p];
#pragma unroll
      for (int e = 0; e < P::W; ++e) wv[p * P::W + e] = (A)q.v[e];
    }
#pragma unroll
    for (int e = 0; e < W; ++e) acc[NV] += wv[e] * wv[e];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      A vk[W];
      IO::load_once(V + (int64_t)k * ldv, g, vk, pol);
#pragma unroll
      for (int e = 0; e < W; ++e) acc[k] += vk[e] * wv[e];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < N - ng * W) {  // the ragged tail, < W elements
    const int64_t i = ng * W + threadIdx.x;
    const A x = (A)w[i];
    acc[NV] += x * x;
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] += IO::template get<A>(V + (int64_t)k * ldv, i) * x;
  }
  block_reduce_store<NV + 1, A>(acc, pp.at());
}

// Decide after a reduction (grid (1, slots)): stage 1 (after pass 1) sets the second-pass
// flag and, without a second pass, 1/h_{j+1,j}; stage 2 (after pass 2) sets 1/h_{j+1,j} from
// the second pass.  Inside the step graph the second pass is the body of an IF node on
// `second` (set_second != 0): stage 1 sets it to 1 for a slot that needs the pass, and stage 2,
// which runs inside that body, sets it back to 0 for the next Arnoldi step of this index and
// counts the body's executions in *passes.
static __global__ void gs_decide_kernel(SlotPtr<double> devp, SlotPtr<float> devfp, int nv,
                                        int stage, const int32_t* run,
                                        cudaGraphConditionalHandle second, int set_second,
                                        unsigned long long* passes) {
  if (stage == 2 && blockIdx.y == 0 && threadIdx.x == 0) {
    if (set_second) cudaGraphSetConditional(second, 0u);
    if (passes) ++*passes;
  }
  if (slot_idle(run)) return;
  double* __restrict__ dev = devp.at();
  float* __restrict__ devf = devfp.at();
  if (threadIdx.x != 0) {
    // FP32 copies of the coefficients this stage produced (threads 1..)
    const int base = stage == 1 ? 0 : kGsH2;
    for (int k = threadIdx.x - 1; k < nv; k += blockDim.x - 1) devf[base + k] = (float)dev[base + k];
    return;
  }
  if (stage == 1) {
    const double nw2 = dev[nv];
    double s = 0.0;
    for (int k = 0; k < nv; ++k) s += dev[k] * dev[k];
    const double est = nw2 - s;
    const bool reorth = !(est > kReorthTheta2 * nw2);
    dev[kGsFlag] = reorth ? 1.0 : 0.0;
    if (reorth && set_second) cudaGraphSetConditional(second, 1u);
    const double hn = reorth ? 0.0 : sqrt(est);
    dev[kGsNorm] = hn;
    dev[kGsInv] = hn > 0.0 ? 1.0 / hn : 0.0;
    devf[kGsFlag] = reorth ? 1.0f : 0.0f;
    devf[kGsInv] = (float)dev[kGsInv];
  } else {
    if (dev[kGsFlag] == 0.0) return;
    const double nw2 = dev[kGsH2 + nv];
    double s = 0.0;
    for (int k = 0; k < nv; ++k) s += dev[kGsH2 + k] * dev[kGsH2 + k];
    const double e2 = nw2 - s;
    const double hn = e2 > 0.0 ? sqrt(e2) : 0.0;
    dev[kGsNorm] = hn;
    dev[kGsInv] = hn > 0.0 ? 1.0 / hn : 0.0;
    devf[kGsInv] = (float)dev[kGsInv];
  }
}

enum GsMode { GS_FINAL1 = 0, GS_REORTH = 1, GS_FINAL2 = 2 };

// FINAL1 / FINAL2: out = (w - sum_k c_k V_k) * dev[kGsInv] with c = h (FINAL1, runs without
// a second pass) or h2 (FINAL2, runs with one); with an FP16 basis the new vector also goes to
// outx in T (the preconditioner's input).  REORTH: w -= sum_k h_k V_k in place, with partial
// V_k . w (rows k < NV) and |w|^2 (row NV) of the result.
template <class T, class B, int NV, int MODE>
__global__ void __launch_bounds__(256) gs_update_kernel(SlotPtr<B> outp, SlotPtr<T> outxp,
                                                        SlotPtr<T> wp, SlotPtr<const B> Vp,
                                                        int64_t ldv, SlotPtr<const double> devp,
                                                        SlotPtr<const float> devfp, int64_t N,
                                                        SlotPtr<double> pp, const int32_t* run) {
  if (slot_idle(run)) return;
  typedef typename AccType<T>::type A;
  typedef Pack16<T> P;
  typedef BasisIO<T, B> IO;
  constexpr int W = IO::W;      // entries per granule
  constexpr int NP = W / P::W;  // 16-byte vector packs per granule
  constexpr bool kCopy = !std::is_same<T, B>::value;
  const A* cf = gs_coef<A>(devp.at(), devfp.at());
  const bool second = cf[kGsFlag] != A(0);
  const bool runs = MODE == GS_FINAL1 ? !second : second;
  if (!runs) return;
  const A* coef = MODE == GS_FINAL2 ? cf + kGsH2 : cf;
  const A inv = cf[kGsInv];
  if (MODE != GS_REORTH && inv == A(0)) return;  // h_{j+1,j} = 0: V_{j+1} is not used
  const B* __restrict__ V = Vp.at();
  T* w = wp.at();
  B* out = MODE == GS_REORTH ? nullptr : outp.at();
  T* outx = kCopy && MODE != GS_REORTH ? outxp.at() : nullptr;
  const uint64_t pol = l2_evict_first();
  A c[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) c[k] = coef[k];
  constexpr int NA = MODE == GS_REORTH ? NV + 1 : 1;
  A acc[NA];
#pragma unroll
  for (int k = 0; k < NA; ++k) acc[k] = A(0);
  const int64_t ng = N / W;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ng;
       g += (int64_t)gridDim.x * blockDim.x) {
    A x[W];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const P q = reinterpret_cast<const P*>(w)[g * NP + p];
#pragma unroll
      for (int e = 0; e < P::W; ++e) x[p * P::W + e] = (A)q.v[e];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      A vk[W];
      // evict_first except in the second pass, which reads V again in the same loop
      if constexpr (MODE == GS_REORTH) IO::load(V + (int64_t)k * ldv, g, vk);
      else IO::load_once(V + (int64_t)k * ldv, g, vk, pol);
#pragma unroll
      for (int e = 0; e < W; ++e) x[e] -= c[k] * vk[e];
    }
    if (MODE == GS_REORTH) {
      A xr[W];
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        P o;
#pragma unroll
        for (int e = 0; e < P::W; ++e) {
          o.v[e] = (T)x[p * P::W + e];
          xr[p * P::W + e] = (A)o.v[e];
        }
        reinterpret_cast<P*>(w)[g * NP + p] = o;
      }
#pragma unroll
      for (int e = 0; e < W; ++e) acc[NV] += xr[e] * xr[e];
      // the second pass is rare: V is read again (from L2) for its dot products rather than
      // held in registers
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        A vk[W];
        IO::load(V + (int64_t)k * ldv, g, vk);
#pragma unroll
        for (int e = 0; e < W; ++e) acc[k] += vk[e] * xr[e];
      }
    } else {
      A y[W];
#pragma unroll
      for (int e = 0; e < W; ++e) y[e] = (A)(T)(x[e] * inv);
      IO::store(out, g, y);
      if (kCopy) {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          P o;
#pragma unroll
          for (int e = 0; e < P::W; ++e) o.v[e] = (T)y[p * P::W + e];
          reinterpret_cast<P*>(outx)[g * NP + p] = o;
        }
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < N - ng * W) {  // the ragged tail
    const int64_t i = ng * W + threadIdx.x;
    A x = (A)w[i];
#pragma unroll
    for (int k = 0; k < NV; ++k) x -= c[k] * IO::template get<A>(V + (int64_t)k * ldv, i);
    if (MODE == GS_REORTH) {
      const T xt = (T)x;
      w[i] = xt;
      acc[NV] += (A)xt * (A)xt;
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] += IO::template get<A>(V + (int64_t)k * ldv, i) * (A)xt;
    } else {
      const T y = (T)(x * inv);
      IO::template set<A>(out, i, (A)y);
      if (kCopy) outx[i] = y;
    }
  }
  if (MODE == GS_REORTH) block_reduce_store<NA, A>(acc, pp.at());
}

// Launch helpers dispatching the vector count to a compile-time constant (1..32).
#define BES_NV_CASES(X) \
  X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) \
  X(17) X(18) X(19) X(20) X(21) X(22) X(23) X(24) X(25) X(26) X(27) X(28) X(29) X(30) X(31) X(32)

template <class T, class B>
void launch_gs_dots(int nvec, dim3 grid, cudaStream_t s, SlotPtr<const B> V, int64_t ldv,
                    SlotPtr<const T> w, int64_t N, SlotPtr<double> partials, const int32_t* run) {
  switch (nvec) {
#define BES_DOTS_CASE(n) \
  case n: gs_dots_kernel<T, B, n><<<grid, 256, 0, s>>>(V, ldv, w, N, partials, run); break;
    BES_NV_CASES(BES_DOTS_CASE)
#undef BES_DOTS_CASE
    default: break;
  }
}

template <class T, class B, int MODE>
void launch_gs_update(int nvec, dim3 grid, cudaStream_t s, SlotPtr<B> out, SlotPtr<T> outx,
                      SlotPtr<T> w, SlotPtr<const B> V, int64_t ldv, SlotPtr<const double> dev,
                      SlotPtr<const float> devf, int64_t N, SlotPtr<double> partials,
                      const int32_t* run) {
  switch (nvec) {
#define BES_UPD_CASE(n)                                                                      \
  case n:                                                                                    \
    gs_update_kernel<T, B, n, MODE><<<grid, 256, 0, s>>>(out, outx, w, V, ldv, dev, devf, N, \
                                                         partials, run);                     \
    break;
    BES_NV_CASES(BES_UPD_CASE)
#undef BES_UPD_CASE
    default: break;
  }
}

// ---- vector kernels --------------------------------------------------------------------------

// out = sum_k y_k V_k over the slot's jc Arnoldi vectors of this cycle
template <class T, class B>
__global__ void __launch_bounds__(256) lincomb_kernel(SlotPtr<T> outp, SlotPtr<const B> Vp,
                                                      int64_t ldv, const int32_t* __restrict__ jc,
                                                      SlotPtr<const double> yp, int64_t N,
                                                      const int32_t* run) {
  if (slot_idle(run)) return;
  typedef typename AccType<T>::type A;
  T* __restrict__ out = outp.at();
  const B* __restrict__ V = Vp.at();
  const int nvec = jc[blockIdx.y];
  __shared__ A ys[kMaxRestart];
  for (int k = threadIdx.x; k < nvec; k += blockDim.x) ys[k] = (A)yp.at()[k];
  __syncthreads();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x) {
    A x = A(0);
    for (int k = 0; k < nvec; ++k) x += ys[k] * BasisIO<T, B>::template get<A>(V + (int64_t)k * ldv, idx);
    out[idx] = (T)x;
  }
}

// First basis vector V_0 = r / beta (r: the right-hand side at the start of a solve, the
// residual at a restart), in the basis's format; with an FP16 basis also its FP32 copy x0
// (the preconditioner's input).  s = the slot's 1/beta (sc[3]).
template <class T, class B>
__global__ void __launch_bounds__(256) basis_start_kernel(SlotPtr<B> V0p, SlotPtr<T> x0p,
                                                          SlotPtr<const T> rp,
                                                          SlotPtr<const double> scp, int64_t N,
                                                          const int32_t* run) {
  if (slot_idle(run)) return;
  typedef typename AccType<T>::type A;
  constexpr bool kCopy = !std::is_same<T, B>::value;
  B* __restrict__ V0 = V0p.at();
  const T* __restrict__ r = rp.at();
  const A s = (A)scp.at()[3];
  T* x0 = kCopy ? x0p.at() : nullptr;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const T y = (T)((A)r[idx] * s);
    BasisIO<T, B>::template set<A>(V0, idx, (A)y);
    if (kCopy) x0[idx] = y;
  }
}

// x += z
template <class T>
__global__ void __launch_bounds__(256) add_kernel(SlotPtr<T> xp, SlotPtr<const T> zp, int64_t N,
                                                  const int32_t* run) {
  if (slot_idle(run)) return;
  T* __restrict__ x = xp.at();
  const T* __restrict__ z = zp.at();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x)
    x[idx] += z[idx];
}

// partial |x|^2 (one value per block)
template <class T>
__global__ void __launch_bounds__(256) norm2_kernel(SlotPtr<const T> xp, int64_t N,
                                                    SlotPtr<double> pp, const int32_t* run) {
  if (slot_idle(run)) return;
  __shared__ double sh[8];
  typedef typename AccType<T>::type A;
  const T* __restrict__ x = xp.at();
  A sa = A(0);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x)
    sa += (A)x[idx] * (A)x[idx];
  const double s = (double)warp_sum_t<A>(sa);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < 8 ? sh[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) pp.at()[blockIdx.x] = v;
  }
}

template <class T>
__global__ void __launch_bounds__(256) zero_kernel(SlotPtr<T> xp, int64_t N, const int32_t* run) {
  if (slot_idle(run)) return;
  T* __restrict__ x = xp.at();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x)
    x[idx] = T(0);
}

// state update W += dW (SolverImplicit::updateSolution_, src/SolverImplicit.cpp:509-528), for
// every slot that took the step; skipped entirely when a face flux was NaN (the step fails)
template <class T>
__global__ void __launch_bounds__(256) state_update_kernel(SlotPtr<double> Up, SlotPtr<const T> dWp,
                                                           int64_t nc, const int* nan_flag,
                                                           const int32_t* run) {
  if (slot_idle(run) || *nan_flag) return;
  // U is [5][nc] (the solver's layout), dW cell-major [nc][5] (the Krylov layout)
  double* __restrict__ U = Up.at();
  const T* __restrict__ dW = dWp.at();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < 5 * nc;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = idx / nc, i = idx - v * nc;
    U[idx] += (double)dW[i * 5 + v];
  }
}

// ---- GMRES control on the device -------------------------------------------------------------
// Right-preconditioned GMRES(m) with x0 = 0 that stops when |g_{j+1}| <= tol |b| (AMGCL
// gmres.hpp:163,214 semantics; the reference's LINEAR_SOLVER_ABS_TOL is relative, quirk Q12),
// for every slot at once.  These kernels run as one block with one thread per slot.  The
// step graph runs a WHILE node over restart cycles whose body holds one IF node per Arnoldi
// step; the kernels below set the nodes' conditions (cudaGraphSetConditional) from the slots'
// flags: a cycle stops when every slot's cycle has stopped, the loop when every slot's solve
// has.  Termination does not depend on convergence: every cycle of a running slot does at
// least one Arnoldi step and the solve stops at linear_solver_max_iter steps, and a slot is
// also stopped (status BES_ERR_TIMEOUT) after a fixed number of restart cycles.

constexpr int kMaxSlots = 256;  // conditions of one implicit context (one control thread each)

struct SlotHandles {
  cudaGraphConditionalHandle h[kMaxSlots];  // IF of each slot's assembly and factorisation
};

struct GmresParam {
  int mr;         // restart length
  int maxiter;    // linear iteration limit
  double tol;     // relative tolerance
};

struct GmresHandles {
  cudaGraphConditionalHandle loop;              // WHILE over restart cycles
  cudaGraphConditionalHandle arn[kMaxRestart];  // IF of Arnoldi step j
  cudaGraphConditionalHandle gs2[kMaxRestart];  // IF of step j's second Gram-Schmidt pass
  int on;                                       // 0: not inside a conditional graph
};

constexpr int kHsize = (kMaxRestart + 1) * kHld;  // Hessenberg entries per slot

__device__ __forceinline__ void set_arnoldi_handles(const GmresHandles& h, int from, int mr,
                                                    unsigned first) {
  if (!h.on) return;
  for (int k = from; k < mr; ++k) cudaGraphSetConditional(h.arn[k], k == from ? first : 0u);
}

// Start of a solve: |b| (reduced into dev[kGsR]) gives beta; slots whose solve runs get
// g = (beta, 0, ...), 1/beta for V_0 = b / beta, and both flags.
static __global__ void gmres_init_kernel(GmresDev g, GmresParam P, GmresHandles h, int nslot,
                                         const int32_t* __restrict__ act,
                                         const int* __restrict__ nan_flag) {
  const int t = threadIdx.x;
  int lin = 0;
  if (t < nslot && act[t]) {
    const double nb = sqrt(g.dev[(int64_t)t * kGsLd + kGsR]);
    const double eps = P.tol * nb;
    double* sc = g.sc + 8 * t;
    sc[0] = nb;
    sc[1] = eps;
    sc[2] = nb;
    sc[3] = nb > 0.0 ? 1.0 / nb : 0.0;
    sc[4] = nb;
    lin = (*nan_flag == 0 && nb > 0.0 && !(nb < eps) && P.maxiter > 0) ? 1 : 0;
    // the reference's solver reports a relative residual of 0 for b = 0; a solve that stops
    // before its first iteration keeps r = b
    sc[5] = nb > 0.0 ? 1.0 : 0.0;
    g.iter[t] = 0;
    g.jc[t] = 0;
    g.second[t] = 0;
    g.status[t] = BES_OK;
    g.cycles[t] = 0;
    double* gg = g.g + (int64_t)t * (kMaxRestart + 1);
    gg[0] = nb;
    for (int k = 1; k <= P.mr; ++k) gg[k] = 0.0;
  }
  if (t < nslot) {
    g.lin[t] = lin;
    g.cyc[t] = lin;
  }
  const int any = __syncthreads_or(lin);
  if (t == 0 && h.on) {
    cudaGraphSetConditional(h.loop, any ? 1u : 0u);
    set_arnoldi_handles(h, 0, P.mr, any ? 1u : 0u);
  }
}

// Arnoldi step j, after the Gram-Schmidt kernels: column j of the Hessenberg matrix from the
// slot's coefficients, the earlier Givens rotations applied to it, a new rotation that zeroes
// h_{j+1,j}, and the rotated right-hand side; the slot's cycle stops when |g_{j+1}| <= eps,
// at the restart length, or at the iteration limit.  Rotation arithmetic without FMA
// contraction.
static __global__ void gmres_givens_kernel(GmresDev g, GmresParam P, GmresHandles h, int nslot,
                                           int j) {
  const int t = threadIdx.x;
  int cont = 0;
  if (t < nslot && g.cyc[t]) {
    double* H = g.H + (int64_t)t * kHsize;
    double* cs = g.cs + (int64_t)t * kMaxRestart;
    double* sn = g.sn + (int64_t)t * kMaxRestart;
    double* gg = g.g + (int64_t)t * (kMaxRestart + 1);
    const double* dev = g.dev + (int64_t)t * kGsLd;
    const bool second = dev[kGsFlag] != 0.0;
    if (second) ++g.second[t];
    for (int i = 0; i <= j; ++i) H[i * kHld + j] = second ? __dadd_rn(dev[i], dev[kGsH2 + i]) : dev[i];
    H[(j + 1) * kHld + j] = dev[kGsNorm];
    for (int i = 0; i < j; ++i) {
      const double a = H[i * kHld + j], b = H[(i + 1) * kHld + j];
      H[i * kHld + j] = __dadd_rn(__dmul_rn(cs[i], a), __dmul_rn(sn[i], b));
      H[(i + 1) * kHld + j] = __dadd_rn(__dmul_rn(-sn[i], a), __dmul_rn(cs[i], b));
    }
    const double a = H[j * kHld + j], c = H[(j + 1) * kHld + j];
    const double d = sqrt(__dadd_rn(__dmul_rn(a, a), __dmul_rn(c, c)));
    cs[j] = d == 0.0 ? 1.0 : a / d;
    sn[j] = d == 0.0 ? 0.0 : c / d;
    H[j * kHld + j] = d;
    H[(j + 1) * kHld + j] = 0.0;
    gg[j + 1] = __dmul_rn(-sn[j], gg[j]);
    gg[j] = __dmul_rn(cs[j], gg[j]);
    g.jc[t] = j + 1;
    const int it = ++g.iter[t];
    cont = (!(fabs(gg[j + 1]) <= g.sc[8 * t + 1]) && j + 1 < P.mr && it < P.maxiter) ? 1 : 0;
    g.cyc[t] = cont;
  }
  const int any = __syncthreads_or(cont);
  if (t == 0) ++g.counters[0];
  if (t == 0 && j + 1 < P.mr) set_arnoldi_handles(h, j + 1, P.mr, any ? 1u : 0u);
}

// End of a cycle: y = H^{-1} g by back substitution over the slot's jc columns.
static __global__ void gmres_solve_y_kernel(GmresDev g, int nslot) {
  const int t = threadIdx.x;
  if (t >= nslot || !g.lin[t]) return;
  const double* H = g.H + (int64_t)t * kHsize;
  const double* gg = g.g + (int64_t)t * (kMaxRestart + 1);
  double* y = g.y + (int64_t)t * kMaxRestart;
  const int j = g.jc[t];
  for (int i = j - 1; i >= 0; --i) {
    double s = gg[i];
    for (int k = i + 1; k < j; ++k) s = __dsub_rn(s, __dmul_rn(H[i * kHld + k], y[k]));
    y[i] = s / H[i * kHld + i];
  }
}

// After x += M^{-1} V y and r = b - A x (|r|^2 reduced into dev[kGsR]): the slot's solve
// stops at |r| <= eps or at the iteration limit; otherwise the next cycle starts from
// V_0 = r / |r|.  guard: restart cycles after which a slot is stopped with BES_ERR_TIMEOUT
// (<= 0: linear_solver_max_iter + 1, more than a running solve can take).
static __global__ void gmres_restart_kernel(GmresDev g, GmresParam P, GmresHandles h, int nslot,
                                            const int32_t* __restrict__ guard) {
  const int t = threadIdx.x;
  int lin = 0;
  if (t < nslot && g.lin[t]) {
    double* sc = g.sc + 8 * t;
    const double nr = sqrt(g.dev[(int64_t)t * kGsLd + kGsR]);
    sc[4] = nr;
    const int limit = *guard > 0 ? *guard : P.maxiter + 1;
    const int cycles = ++g.cycles[t];
    if (nr <= sc[1] || g.iter[t] >= P.maxiter) {
      sc[5] = nr / sc[0];
    } else if (cycles >= limit) {
      sc[5] = nr / sc[0];
      g.status[t] = BES_ERR_TIMEOUT;
    } else {
      sc[2] = nr;
      sc[3] = 1.0 / nr;
      double* gg = g.g + (int64_t)t * (kMaxRestart + 1);
      gg[0] = nr;
      for (int k = 1; k <= P.mr; ++k) gg[k] = 0.0;
      g.jc[t] = 0;
      lin = 1;
    }
    g.lin[t] = lin;
    g.cyc[t] = lin;
  }
  const int any = __syncthreads_or(lin);
  if (t == 0) ++g.counters[1];
  if (t == 0 && h.on) {
    cudaGraphSetConditional(h.loop, any ? 1u : 0u);
    set_arnoldi_handles(h, 0, P.mr, any ? 1u : 0u);
  }
}

// End of the step: what the host reads back per slot.
static __global__ void gmres_finish_kernel(GmresDev g, StepResult* __restrict__ res, int nslot,
                                           const int32_t* __restrict__ act) {
  const int t = threadIdx.x;
  if (t >= nslot) return;
  const int a = act[t] != 0;
  res[t].active = a;
  res[t].iters = a ? g.iter[t] : 0;
  res[t].second = a ? g.second[t] : 0;
  res[t].status = a ? g.status[t] : BES_OK;
  res[t].rel = a ? g.sc[8 * t + 5] : 0.0;
}

// Start of a step: the assembly IF node of every slot runs only for slots that take the step;
// each slot's global time step starts from +inf.
static __global__ void step_begin_kernel(SlotHandles hs, int on, int nslot,
                                         const int32_t* __restrict__ act,
                                         unsigned long long* __restrict__ dtmin) {
  for (int t = threadIdx.x; t < nslot; t += blockDim.x) {
    dtmin[t] = (unsigned long long)__double_as_longlong(1e300);
    if (on) cudaGraphSetConditional(hs.h[t], act[t] ? 1u : 0u);
  }
}

// Profiling: the global nanosecond timer before (begin) and after a category's work; P holds
// the open stamp [PROF_NCAT], the accumulated nanoseconds [PROF_NCAT] and the counts.
static __global__ void prof_stamp_kernel(unsigned long long* P, int cat, int begin) {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  if (begin) {
    P[cat] = t;
  } else {
    P[PROF_NCAT + cat] += t - P[cat];
    P[2 * PROF_NCAT + cat] += 1;
  }
}

}  // namespace bes
