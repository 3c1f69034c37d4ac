// Kernels of the implicit (backward-Euler) path: first-order flux Jacobians, assembly of
// the 5x5-block system in ELL form, block-Jacobi and colour-ordered block-ILU(0)
// preconditioners, and the vector kernels of restarted GMRES.  T is the precision of the
// matrix, preconditioner and Krylov vectors (double for the plain method, float for the
// defect correction); residuals, right-hand sides and the state stay FP64.
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

// forward solve of one colour: out_i = in_i - sum_{lower j} L_ij out_j
template <class T>
__global__ void __launch_bounds__(128) ilu_lower_kernel(DevMesh m, const int32_t* __restrict__ rows,
                                                        int nrows, const int32_t* __restrict__ pos,
                                                        const T* __restrict__ A,
                                                        const T* in, T* out) {  // may alias
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  const int nc = m.nc;
  const int i = rows[t];
  const int pi = pos[i];
  T acc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = in[(int64_t)i * 5 + v];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int j = m.adj[s * nc + i];
    if (j < 0 || pos[j] >= pi) continue;
    T y[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) y[v] = out[(int64_t)j * 5 + v];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] -= ellc(A, 1 + s, r * 5 + c, nc, i) * y[c];
  }
#pragma unroll
  for (int v = 0; v < 5; ++v) out[(int64_t)i * 5 + v] = acc[v];
}

// backward solve of one colour, in place: z_i = inv(U_ii) (y_i - sum_{upper k} U_ik z_k)
template <class T>
__global__ void __launch_bounds__(128) ilu_upper_kernel(DevMesh m, const int32_t* __restrict__ rows,
                                                        int nrows, const int32_t* __restrict__ pos,
                                                        const T* __restrict__ A,
                                                        const T* __restrict__ Dinv, T* __restrict__ z) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows) return;
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

// Colour-ordered block-ILU(0) sweep when the colours are contiguous cell ranges in increasing
// order (the colour-major numbering): the rows of one colour are [r0, r1), lower neighbours
// are j < r0 and upper neighbours k >= r1, so no row list or position lookup is needed.  The
// lower solve of colour 0 is the identity, so its y values are read from `in` where they are
// needed (lower neighbours in [0, s1), colour 0's own upper solve) instead of being copied.
//   LOWER only        colours 1..C-2 of the forward sweep: out_i = in_i - sum L_ij y_j
//   LOWER and UPPER   the last colour: both solves at once (it has no upper neighbours)
//   UPPER only        colours C-2..0 of the backward sweep: out_i = inv(U_ii)(y_i - sum U_ik z_k)
// `in` and `out` must not alias.
template <class T, bool LOWER, bool UPPER>
__global__ void __launch_bounds__(128) ilu_colour_kernel(DevMesh m, int r0, int r1, int s1,
                                                         const T* __restrict__ A,
                                                         const T* __restrict__ Dinv,
                                                         const T* __restrict__ in,
                                                         T* __restrict__ out) {
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  const int nc = m.nc;
  const T* own = (LOWER || r0 == 0) ? in : out;
  T acc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = own[(int64_t)i * 5 + v];
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int j = m.adj[s * nc + i];
    const bool lower = LOWER && j >= 0 && j < r0;
    const bool upper = UPPER && j >= r1;
    if (!lower && !upper) continue;
    const T* src = (lower && j < s1) ? in : out;
    T y[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) y[v] = src[(int64_t)j * 5 + v];
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

// block-Jacobi application: out_i = Dinv_i in_i
template <class T>
__global__ void __launch_bounds__(256) jacobi_apply_kernel(int nc, const T* __restrict__ Dinv,
                                                           const T* __restrict__ in,
                                                           T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
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

// y = A x (ELL), optionally y = b - A x
template <class T>
__global__ void __launch_bounds__(256) spmv_kernel(DevMesh m, const T* __restrict__ A,
                                                   const T* __restrict__ x,
                                                   const T* __restrict__ b, T* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = m.nc;
  if (i >= nc) return;
  T acc[5], xi[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) xi[v] = x[(int64_t)i * 5 + v];
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
#pragma unroll
    for (int v = 0; v < 5; ++v) xi[v] = x[(int64_t)j * 5 + v];
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] += ellc(A, 1 + q, r * 5 + c, nc, i) * xi[c];
  }
#pragma unroll
  for (int r = 0; r < 5; ++r)
    y[(int64_t)i * 5 + r] = b ? b[(int64_t)i * 5 + r] - acc[r] : acc[r];
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

// y = A x (or b - A x) with A in packed form: per block, the neighbour's values are scaled
// by the block's scale and multiplied by the 16-bit entries
static __global__ void __launch_bounds__(256) spmv_packed_kernel(
    DevMesh m, const __half2* __restrict__ H, const float* __restrict__ S,
    const float* __restrict__ x, const float* __restrict__ b, float* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nc = m.nc;
  if (i >= nc) return;
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
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const float sc = S[(int64_t)s * nc + i];
    float xs[5], a[26];
#pragma unroll
    for (int v = 0; v < 5; ++v) xs[v] = sc * x[(int64_t)jn[s] * 5 + v];
    load_packed(H, s, nc, i, a);
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] = fmaf(a[r * 5 + c], xs[c], acc[r]);
  }
#pragma unroll
  for (int r = 0; r < 5; ++r)
    y[(int64_t)i * 5 + r] = b ? b[(int64_t)i * 5 + r] - acc[r] : acc[r];
}

// ilu_colour_kernel with packed factors: L / U blocks in H slots 0..3 (local faces 0..3),
// inv(U_ii) in D (one slot)
template <bool LOWER, bool UPPER>
__global__ void __launch_bounds__(128) ilu_colour_packed_kernel(
    DevMesh m, int r0, int r1, int s1, const __half2* __restrict__ H, const float* __restrict__ HS,
    const __half2* __restrict__ D, const float* __restrict__ DS, const float* __restrict__ in,
    float* __restrict__ out) {
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  const int nc = m.nc;
  const float* own = (LOWER || r0 == 0) ? in : out;
  float acc[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) acc[v] = own[(int64_t)i * 5 + v];
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
    const float sc = HS[(int64_t)s * nc + i];
    float y[5], a[26];
#pragma unroll
    for (int v = 0; v < 5; ++v) y[v] = sc * src[(int64_t)j * 5 + v];
    load_packed(H, s, nc, i, a);
#pragma unroll
    for (int r = 0; r < 5; ++r)
#pragma unroll
      for (int c = 0; c < 5; ++c) acc[r] = fmaf(-a[r * 5 + c], y[c], acc[r]);
  }
  if (UPPER) {
    float a[26];
    load_packed(D, 0, nc, i, a);
    const float sc = DS[i];
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

// block-Jacobi application with a packed inverse diagonal
static __global__ void __launch_bounds__(256) jacobi_apply_packed_kernel(
    int nc, const __half2* __restrict__ D, const float* __restrict__ DS,
    const float* __restrict__ in, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  float x[5], a[26];
#pragma unroll
  for (int v = 0; v < 5; ++v) x[v] = in[(int64_t)i * 5 + v];
  load_packed(D, 0, nc, i, a);
  const float sc = DS[i];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c < 5; ++c) acc = fmaf(a[r * 5 + c], x[c], acc);
    out[(int64_t)i * 5 + r] = sc * acc;
  }
}

// Per-thread accumulation type of the vector kernels: the FP32 system accumulates each
// thread's few elements in FP32 (the FP64 pipe is ~60x slower on this GPU) and reduces
// across threads and blocks in FP64; the FP64 system stays FP64 throughout.
template <class T> struct AccType { typedef double type; };
template <> struct AccType<float> { typedef float type; };

// Warp sum in the accumulation type (FP32 for the FP32 system: FP64 arithmetic, conversions
// included, runs on the FP64 pipe, which is ~60x slower on this GPU).
template <class A>
__device__ __forceinline__ A warp_sum_t(A x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Block reduction of NV per-thread accumulators; partials[k*gridDim + blk] (FP64).  Lanes are
// summed in the accumulation type; each warp's sum is widened to FP64 once and the block's
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

// ---- Gram-Schmidt of the Arnoldi step -------------------------------------------------
// Classical Gram-Schmidt with a conditional second pass (the oracle's linsolve.hpp gmres
// states the same algorithm):
//   pass 1   h = V^T w and |w|^2 in one read of V and w (gs_dots_kernel);
//   decide   |w - V h|^2 = |w|^2 - |h|^2 (Pythagoras); a second pass runs only when this
//            is <= kReorthTheta2 |w|^2 (gs_decide_kernel, on the device, so the host is not
//            asked);
//   no second pass: V_{j+1} = (w - V h) / sqrt(|w|^2 - |h|^2) in one more read of V and w
//            (gs_update_kernel<FINAL1>);
//   second pass: w -= V h with V^T w and |w|^2 of the result in the same read
//            (gs_update_kernel<REORTH>), then V_{j+1} = (w - V h2) / norm (<FINAL2>).
// The kernels of the path not taken return at once.  Device scalars (dev = red_out):
//   dev[0..nv-1] h, dev[nv] |w|^2; dev[kGsH2 + k] h2, dev[kGsH2 + nv] |w'|^2;
//   dev[kGsFlag] 1 if the second pass runs, dev[kGsInv] 1/h_{j+1,j} (0: leave V_{j+1}),
//   dev[kGsNorm] h_{j+1,j}.
//   devf: FP32 copies of h, h2, the flag and 1/h_{j+1,j} at the same offsets, written by
//   gs_decide_kernel, so that FP32 update kernels convert nothing per thread.
constexpr double kReorthTheta2 = 1.0 / 16.0;
constexpr int kGsH2 = 40, kGsFlag = 80, kGsInv = 81, kGsNorm = 82, kGsScalars = 83;

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

// 16-byte unit of the vector kernels; the Krylov basis stride is a multiple of it
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
    const uint4 u = reinterpret_cast<const uint4*>(V)[g];
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
__global__ void __launch_bounds__(256) gs_dots_kernel(const B* __restrict__ V, int64_t ldv,
                                                      const T* __restrict__ w, int64_t N,
                                                      double* __restrict__ partials) {
  typedef typename AccType<T>::type A;
  typedef Pack16<T> P;
  typedef BasisIO<T, B> IO;
  constexpr int W = IO::W;      // entries per granule
  constexpr int NP = W / P::W;  // 16-byte vector packs per granule
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
      IO::load(V + (int64_t)k * ldv, g, vk);
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
  block_reduce_store<NV + 1, A>(acc, partials);
}

// Decide after a reduction: stage 1 (after pass 1) sets the second-pass flag and, without a
// second pass, 1/h_{j+1,j}; stage 2 (after pass 2) sets 1/h_{j+1,j} from the second pass.
static __global__ void gs_decide_kernel(double* __restrict__ dev, float* __restrict__ devf,
                                        int nv, int stage) {
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
__global__ void __launch_bounds__(256) gs_update_kernel(B* __restrict__ out, T* __restrict__ outx,
                                                        T* w, const B* __restrict__ V, int64_t ldv,
                                                        const double* __restrict__ dev,
                                                        const float* __restrict__ devf,
                                                        int64_t N, double* __restrict__ partials) {
  typedef typename AccType<T>::type A;
  typedef Pack16<T> P;
  typedef BasisIO<T, B> IO;
  constexpr int W = IO::W;      // entries per granule
  constexpr int NP = W / P::W;  // 16-byte vector packs per granule
  constexpr bool kCopy = !std::is_same<T, B>::value;
  const A* cf = gs_coef<A>(dev, devf);
  const bool second = cf[kGsFlag] != A(0);
  const bool runs = MODE == GS_FINAL1 ? !second : second;
  if (!runs) return;
  const A* coef = MODE == GS_FINAL2 ? cf + kGsH2 : cf;
  const A inv = cf[kGsInv];
  if (MODE != GS_REORTH && inv == A(0)) return;  // h_{j+1,j} = 0: V_{j+1} is not used
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
      IO::load(V + (int64_t)k * ldv, g, vk);
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
  if (MODE == GS_REORTH) block_reduce_store<NA, A>(acc, partials);
}

// Launch helpers dispatching the vector count to a compile-time constant (1..32).
#define BES_NV_CASES(X) \
  X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) \
  X(17) X(18) X(19) X(20) X(21) X(22) X(23) X(24) X(25) X(26) X(27) X(28) X(29) X(30) X(31) X(32)

template <class T, class B>
void launch_gs_dots(int nvec, int G, cudaStream_t s, const B* V, int64_t ldv, const T* w,
                    int64_t N, double* partials) {
  switch (nvec) {
#define BES_DOTS_CASE(n) \
  case n: gs_dots_kernel<T, B, n><<<G, 256, 0, s>>>(V, ldv, w, N, partials); break;
    BES_NV_CASES(BES_DOTS_CASE)
#undef BES_DOTS_CASE
    default: break;
  }
}

template <class T, class B, int MODE>
void launch_gs_update(int nvec, int G, cudaStream_t s, B* out, T* outx, T* w, const B* V,
                      int64_t ldv, const double* dev, const float* devf, int64_t N,
                      double* partials) {
  switch (nvec) {
#define BES_UPD_CASE(n) \
  case n: gs_update_kernel<T, B, n, MODE><<<G, 256, 0, s>>>(out, outx, w, V, ldv, dev, devf, N, partials); break;
    BES_NV_CASES(BES_UPD_CASE)
#undef BES_UPD_CASE
    default: break;
  }
}

template <class T>
__global__ void __launch_bounds__(256) scale_kernel(T* __restrict__ out, const T* __restrict__ in,
                                                    double s, int64_t N) {
  typedef typename AccType<T>::type A;
  const A sa = (A)s;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x)
    out[idx] = (T)((A)in[idx] * sa);
}

// out = sum_k y_k V_k
template <class T, class B>
__global__ void __launch_bounds__(256) lincomb_kernel(T* __restrict__ out, const B* __restrict__ V,
                                                      int64_t ldv, int nvec,
                                                      const double* __restrict__ y, int64_t N) {
  typedef typename AccType<T>::type A;
  __shared__ A ys[64];
  for (int k = threadIdx.x; k < nvec; k += blockDim.x) ys[k] = (A)y[k];
  __syncthreads();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x) {
    A x = A(0);
    for (int k = 0; k < nvec; ++k) x += ys[k] * BasisIO<T, B>::template get<A>(V + (int64_t)k * ldv, idx);
    out[idx] = (T)x;
  }
}

// First basis vector from an FP32 residual: V_0 = s r in the basis's format, and its FP32
// copy x0 (the preconditioner's input)
static __global__ void __launch_bounds__(256) basis_start_kernel(__half* __restrict__ V0,
                                                                 float* __restrict__ x0,
                                                                 const float* __restrict__ r,
                                                                 double s, int64_t N) {
  const float sf = (float)s;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const float y = r[idx] * sf;
    x0[idx] = y;
    BasisIO<float, __half>::set<float>(V0, idx, y);
  }
}

// x += z
template <class T>
__global__ void __launch_bounds__(256) add_kernel(T* __restrict__ x, const T* __restrict__ z,
                                                  int64_t N) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x)
    x[idx] += z[idx];
}

// partial |x|^2
template <class T>
__global__ void __launch_bounds__(256) norm2_kernel(const T* __restrict__ x, int64_t N,
                                                    double* __restrict__ partials) {
  __shared__ double sh[8];
  typedef typename AccType<T>::type A;
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
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
  }
}

// state update W += dW (SolverImplicit::updateSolution_, src/SolverImplicit.cpp:509-528)
template <class T>
__global__ void __launch_bounds__(256) state_update_kernel(double* __restrict__ U,
                                                           const T* __restrict__ dW, int64_t nc) {
  // U is [5][nc] (the solver's layout), dW cell-major [nc][5] (the Krylov layout)
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < 5 * nc;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = idx / nc, i = idx - v * nc;
    U[idx] += (double)dW[i * 5 + v];
  }
}

template <class T>
__global__ void __launch_bounds__(256) zero_kernel(T* __restrict__ x, int64_t N) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (int64_t)gridDim.x * blockDim.x)
    x[idx] = T(0);
}

}  // namespace bes
