// Kernels of the implicit (backward-Euler) path: first-order flux Jacobians, assembly of
// the 5x5-block system in ELL form, the block-ILU(0) factorisation and the 16-bit
// block-scaled copies of the system (the Krylov side is in krylov_kernels.cuh).  T is the
// precision of the matrix, preconditioner and Krylov vectors (double for the plain method,
// float for the defect correction); residuals, right-hand sides and the state stay FP64.
//
// ELL layout: value q (= row*5 + col) of slot s of cell i is A[(s*25 + q)*nc + i]; slot 0 is
// the diagonal block, slot 1+m the block coupling to the neighbour across local face m.
// The Krylov-side vectors (right-hand side b, iterates, basis, preconditioner output) are
// cell-major: component v of cell i is x[i*5 + v], so a neighbour's five values are one
// 20-byte gather (SoA would touch five 32-byte sectors) while streams stay coalesced; the
// FP64 state and residual keep the solver's [5][nc] layout.
#pragma once
#include <cuda_fp16.h>

#include <type_traits>

#include "explicit_kernels.cuh"

namespace bes {

constexpr int kRedBlocks = 1024;  // fixed grid of the reduction kernels (deterministic sums)

template <class T>
__device__ __forceinline__ T& ell(T* A, int s, int q, int nc, int i) {
  return A[(int64_t)(s * 25 + q) * nc + i];
}
template <class T>
__device__ __forceinline__ T ellc(const T* A, int s, int q, int nc, int i) {
  return A[(int64_t)(s * 25 + q) * nc + i];
}

// a[k] for a runtime k in [0, 4) without indexing the array (keeps it in registers)
__device__ __forceinline__ int sel4(const int* a, int k) {
  return k == 0 ? a[0] : (k == 1 ? a[1] : (k == 2 ? a[2] : a[3]));
}

// 5x5 inverse by Gauss-Jordan elimination with partial pivoting.
template <class T>
__device__ __forceinline__ void inv5(const T* a, T* inv) {
  T m[5][10];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      m[i][j] = a[i * 5 + j];
      m[i][5 + j] = (i == j) ? T(1) : T(0);
    }
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    // pivot: the first row r >= c with the largest |m[r][c]|; the swap is written with
    // compile-time row indices (predicated), so m stays in registers
    int p = c;
    T best = fabs(m[c][c]);
#pragma unroll
    for (int r = c + 1; r < 5; ++r)
      if (fabs(m[r][c]) > best) {
        best = fabs(m[r][c]);
        p = r;
      }
#pragma unroll
    for (int r = c + 1; r < 5; ++r)
      if (r == p)
#pragma unroll
        for (int j = 0; j < 10; ++j) {
          const T t = m[r][j];
          m[r][j] = m[c][j];
          m[c][j] = t;
        }
    const T piv = T(1) / m[c][c];
#pragma unroll
    for (int j = 0; j < 10; ++j) m[c][j] *= piv;
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      if (r == c) continue;
      const T f = m[r][c];
#pragma unroll
      for (int j = 0; j < 10; ++j) m[r][j] -= f * m[c][j];
    }
  }
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int j = 0; j < 5; ++j) inv[i * 5 + j] = m[i][5 + j];
}

// ---------------------------------------------------------------------------------------
// Jacobians and assembly (SolverImplicit::computeFaceFluxes_, src/SolverImplicit.cpp:358-507)
// ---------------------------------------------------------------------------------------
struct FaceLocal {
  const int8_t* m_own;  // local face index of the face in its owner
  const int8_t* m_nb;   // ... in its neighbour (-1 on boundary faces)
};

// Per face: dF/dU_L and dF/dU_R at the FIRST-order states (the two cell averages) by
// forward-mode derivatives of the flux templates (two passes of 5 slots).  Writes the
// face's two off-diagonal blocks (each added `rep` times from zero, as the reference's
// addToBlock sits inside the variable loop, quirk Q9) and its contributions to the two
// diagonal blocks (m_o J_L for the owner, -m_n J_R for the neighbour) for the cell sweep.
template <class T>
__global__ void __launch_bounds__(128) face_jacobian_kernel(
    DevMesh m, Params prm, FaceLocal fl, const double* __restrict__ U,
    const double* __restrict__ dt, const unsigned long long* __restrict__ dtmin, int local_dt,
    int rep, T* __restrict__ A, T* __restrict__ Dc) {
  typedef Dual<5, T> DT;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = m.nc, nf = m.nf;
  if (f >= nf) return;
  const int o = m.fown[f];
  double n[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) n[d] = m.fn[(int64_t)d * nf + f];
  const double area = m.farea[f];
  const double dtg = local_dt ? 0.0 : __longlong_as_double((long long)*dtmin);
  const double m_o = (local_dt ? dt[o] : dtg) * m.inv_vol[o] * area;
  T JL[25], JR[25];
  T ul[5], ur[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) ul[v] = (T)U[(int64_t)v * nc + o];
  const bool interior = f < m.nf_int;
  int nb = -1;
  if (interior) {
    nb = m.fnb[f];
#pragma unroll
    for (int v = 0; v < 5; ++v) ur[v] = (T)U[(int64_t)v * nc + nb];
  }
  GasConst g = prm.gas;
  for (int side = 0; side < (interior ? 2 : 1); ++side) {
    DT dl[5], dr[5], dfl[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      dl[v] = DT(ul[v]);
      dr[v] = DT(interior ? ur[v] : T(0));
      if (side == 0)
        dl[v].d[v] = T(1);
      else
        dr[v].d[v] = T(1);
    }
    if (interior)
      roe_flux(g, dl, dr, n, dfl);
    else if (f < m.nf_int + m.nf_slip)
      slipwall_flux(g, dl, n, dfl);
    else
      freestream_flux(g, dl, prm.pinf_dev, n, dfl);
    T* J = side == 0 ? JL : JR;
#pragma unroll
    for (int a = 0; a < 5; ++a)
#pragma unroll
      for (int b = 0; b < 5; ++b) J[a * 5 + b] = dfl[a].d[b];
  }
  const T mo = (T)m_o;
#pragma unroll
  for (int q = 0; q < 25; ++q) Dc[(int64_t)q * nf + f] = mo * JL[q];
  if (interior) {
    const double m_n = (local_dt ? dt[nb] : dtg) * m.inv_vol[nb] * area;
    const T mn = (T)m_n;
    const int so = 1 + fl.m_own[f], sn = 1 + fl.m_nb[f];
#pragma unroll
    for (int q = 0; q < 25; ++q) {
      Dc[(int64_t)(25 + q) * nf + f] = -mn * JR[q];
      const T yo = mo * JR[q], yn = -mn * JL[q];
      T xo = T(0), xn = T(0);
      for (int r = 0; r < rep; ++r) {
        xo += yo;
        xn += yn;
      }
      ell(A, so, q, nc, o) = xo;
      ell(A, sn, q, nc, nb) = xn;
    }
  }
}

// Per cell: right-hand side -(dt/V) sum(+-F A) in the reference's face order, the diagonal
// block I + rep * sum of the face contributions, block-Jacobi inverse (optional), and block
// partial norms of the right-hand side.
template <class T>
__global__ void __launch_bounds__(128) cell_assemble_kernel(
    DevMesh m, const double* __restrict__ FA, const double* __restrict__ dt,
    const unsigned long long* __restrict__ dtmin, int local_dt, int rep, const T* __restrict__ Dc,
    T* __restrict__ A, T* __restrict__ Dinv, double* __restrict__ rhs, T* __restrict__ rhs_t,
    double* __restrict__ partials) {
  const int nc = m.nc, nf = m.nf;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double b[5] = {0, 0, 0, 0, 0};
  double R[5] = {0, 0, 0, 0, 0};  // unscaled residual sum(+-F A), for convergence monitoring
  if (i < nc) {
    const double dti = local_dt ? dt[i] : __longlong_as_double((long long)*dtmin);
    const double k = dti * m.inv_vol[i];
    T D[25];
#pragma unroll
    for (int q = 0; q < 25; ++q) D[q] = (q % 6 == 0) ? T(1) : T(0);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int gf = m.gface[s * nc + i];
      if (gf == bes::kNoFace) continue;  // empty slot of a triangle
      const int f = gf >= 0 ? gf : ~gf;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double fa = FA[(int64_t)v * nf + f];
        const double x = k * fa;
        b[v] = gf >= 0 ? b[v] - x : b[v] + x;
        R[v] = gf >= 0 ? R[v] + fa : R[v] - fa;
      }
      const T* src = Dc + (gf >= 0 ? 0 : (int64_t)25 * nf);
#pragma unroll
      for (int q = 0; q < 25; ++q) {
        const T y = src[(int64_t)q * nf + f];
        for (int r = 0; r < rep; ++r) D[q] += y;
      }
    }
#pragma unroll
    for (int q = 0; q < 25; ++q) ell(A, 0, q, nc, i) = D[q];
    if (Dinv) {
      T inv[25];
      inv5(D, inv);
#pragma unroll
      for (int q = 0; q < 25; ++q) Dinv[(int64_t)q * nc + i] = inv[q];
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      rhs[(int64_t)v * nc + i] = b[v];
      rhs_t[(int64_t)i * 5 + v] = (T)b[v];
    }
  }
  __shared__ double sh[15][4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    const double s2 = warp_sum(b[v] * b[v]);
    const double mx = warp_max(fabs(b[v]));
    const double r2 = warp_sum(R[v] * R[v]);
    if (lane == 0) {
      sh[v][wid] = s2;
      sh[5 + v][wid] = mx;
      sh[10 + v][wid] = r2;
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int q = 0; q < 15; ++q) {
      double x = lane < 4 ? sh[q][lane] : 0.0;
      x = (q >= 5 && q < 10) ? warp_max(x) : warp_sum(x);
      // rows: 0-4 sum b^2, 5-9 max |b|, 10-14 sum R^2
      const int row = q < 5 ? q : (q < 10 ? q + 5 : q - 5);
      if (lane == 0) partials[(int64_t)row * gridDim.x + blockIdx.x] = x;
    }
  }
}

// Reduce `nvals` rows of per-block partials (sums, or maxima for rows >= nsum) in a fixed
// order; one block per value.  out[k] = sum (sqrt if sqrt_sums) or max.
static __global__ void __launch_bounds__(256) reduce_rows_kernel(const double* __restrict__ partials,
                                                          int nblocks, int nsum, int sqrt_sums,
                                                          double* __restrict__ out) {
  __shared__ double sh[8];
  const int k = blockIdx.x;
  const bool is_sum = k < nsum;
  double x = is_sum ? 0.0 : 0.0;
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
    if (lane == 0) out[k] = (is_sum && sqrt_sums) ? sqrt(x) : x;
  }
}

// Colour-ordered block ILU(0), one colour per launch (rows of one colour are independent).
// IKJ order: the lower blocks of a row are eliminated in increasing factorisation position.
// RANGE: the stage is the contiguous row range [r0, r0 + nrows) and the factorisation
// position is the cell number (colour-major numbering), so no row list or position lookup.
template <class T, bool RANGE = false>
__global__ void __launch_bounds__(128) ilu_factor_kernel(DevMesh m, const int32_t* __restrict__ rows,
                                                         int nrows, const int32_t* __restrict__ pos,
                                                         T* __restrict__ A, T* __restrict__ Dinv,
                                                         int r0 = 0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  const int nc = m.nc;
  const int i = RANGE ? r0 + t : rows[t];
  const int pi = RANGE ? i : pos[i];
  int nbr[4], pn[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    nbr[s] = m.adj[s * nc + i];
    pn[s] = nbr[s] >= 0 ? (RANGE ? nbr[s] : pos[nbr[s]]) : 0x7fffffff;
  }
  // lower slots in increasing position: rank[s] = number of lower slots before slot s (the
  // neighbours are distinct cells, so positions are distinct).  All indexing of nbr / pn / rank
  // uses compile-time indices, so they stay in registers.
  bool low[4];
  int rank[4], nl = 0;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    low[s] = nbr[s] >= 0 && pn[s] < pi;
    nl += low[s];
  }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    rank[s] = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) rank[s] += (low[t] && pn[t] < pn[s]) ? 1 : 0;
  }
  for (int li = 0; li < nl; ++li) {
    int s = 0, j = 0, pj = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (low[t] && rank[t] == li) {
        s = t;
        j = nbr[t];
        pj = pn[t];
      }
    // blocks are loaded into registers before any store: A is read and written through one
    // pointer, so loads issued after a store could not be batched or reused
    T L[25], Ais[25], Dj[25];
#pragma unroll
    for (int q = 0; q < 25; ++q) {
      Ais[q] = ellc(A, 1 + s, q, nc, i);
      Dj[q] = Dinv[(int64_t)q * nc + j];
    }
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < 5; ++k) acc += Ais[r * 5 + k] * Dj[k * 5 + c];
        L[r * 5 + c] = acc;
      }
#pragma unroll
    for (int q = 0; q < 25; ++q) ell(A, 1 + s, q, nc, i) = L[q];
    // A_ik -= L_ij U_jk for every k in row i's pattern with pos(k) > pos(j) and (j,k) present
#pragma unroll 1
    for (int kk = -1; kk < 4; ++kk) {
      const int col = kk < 0 ? i : sel4(nbr, kk);
      if (kk >= 0 && (col < 0 || sel4(pn, kk) <= pj)) continue;
      int sj = -1;
      for (int q = 0; q < 4; ++q)
        if (m.adj[q * nc + j] == col) sj = q;
      if (sj < 0) continue;
      const int dst = kk < 0 ? 0 : 1 + kk;
      T U[25], Ad[25];
#pragma unroll
      for (int q = 0; q < 25; ++q) {
        U[q] = ellc(A, 1 + sj, q, nc, j);
        Ad[q] = ellc(A, dst, q, nc, i);
      }
#pragma unroll
      for (int r = 0; r < 5; ++r)
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          T acc = T(0);
#pragma unroll
          for (int k = 0; k < 5; ++k) acc += L[r * 5 + k] * U[k * 5 + c];
          Ad[r * 5 + c] -= acc;
        }
#pragma unroll
      for (int q = 0; q < 25; ++q) ell(A, dst, q, nc, i) = Ad[q];
    }
  }
}

// inverse of the factored diagonal block of each row of a stage (after ilu_factor_kernel)
template <class T, bool RANGE = false>
__global__ void __launch_bounds__(128) ilu_invert_kernel(DevMesh m, const int32_t* __restrict__ rows,
                                                         int nrows, const T* __restrict__ A,
                                                         T* __restrict__ Dinv, int r0 = 0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  const int nc = m.nc;
  const int i = RANGE ? r0 + t : rows[t];
  T D[25], inv[25];
#pragma unroll
  for (int q = 0; q < 25; ++q) D[q] = ellc(A, 0, q, nc, i);
  inv5(D, inv);
#pragma unroll
  for (int q = 0; q < 25; ++q) Dinv[(int64_t)q * nc + i] = inv[q];
}

// ---- 16-bit block-scaled storage of the FP32 system (precision 2)
// A 5x5 block is stored as 13 half2 words (entries 2p and 2p+1 of the row-major block; the
// 26th half is 0) in the layout H[slot][13][nc], plus one FP32 scale per block S[slot][nc]:
// entry q = S * H[q].  The scale is the smallest power of two >= the block's largest |entry|,
// so the rescaling is exact and every stored entry lies in [-1, 1] with FP16's 11-bit
// significand; entries below 2^-14 of the scale become FP16 subnormals (absolute error at most
// 2^-25 of the scale).  Per block: 52 + 4 bytes instead of 100.

// smallest power of two >= x (x >= 0 and finite); 1 for x == 0
__device__ __forceinline__ float pow2_ceil(float x) {
  if (x == 0.0f) return 1.0f;
  const unsigned b = __float_as_uint(x);
  return __uint_as_float((b + 0x007fffffu) & 0xff800000u);
}

// pack slots [slot0, slot0 + gridDim.y) of a dense ELL array (or a [25][nc] array with
// slot0 = 0) into H / S slots [0, gridDim.y); one thread per (cell, slot)
static __global__ void __launch_bounds__(256) pack_blocks_kernel(const float* __restrict__ A,
                                                                 int slot0, int nc,
                                                                 __half2* __restrict__ H,
                                                                 float* __restrict__ S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  if (i >= nc) return;
  float a[26];
  float mx = 0.0f;
#pragma unroll
  for (int q = 0; q < 25; ++q) {
    a[q] = A[(int64_t)((slot0 + s) * 25 + q) * nc + i];
    mx = fmaxf(mx, fabsf(a[q]));
  }
  a[25] = 0.0f;
  const float sc = pow2_ceil(mx);
  const float inv = 1.0f / sc;  // exact: sc is a power of two
#pragma unroll
  for (int p = 0; p < 13; ++p)
    H[(int64_t)(s * 13 + p) * nc + i] = __floats2half2_rn(a[2 * p] * inv, a[2 * p + 1] * inv);
  S[(int64_t)s * nc + i] = sc;
}

__device__ __forceinline__ void load_packed(const __half2* __restrict__ H, int s, int nc, int i,
                                            float* a) {
#pragma unroll
  for (int p = 0; p < 13; ++p) {
    const float2 f = __half22float2(H[(int64_t)(s * 13 + p) * nc + i]);
    a[2 * p] = f.x;
    a[2 * p + 1] = f.y;
  }
}

}  // namespace bes
