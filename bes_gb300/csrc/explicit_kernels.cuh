// Kernels of the explicit residual/update path (FP64).  One explicit stage is three sweeps:
//   cell_recon_kernel  per cell: Green-Gauss gradient (GradientGreenGauss.cpp:21-135),
//                      Venkatakrishnan limiter (LimiterVenkatakrishnan.cpp:21-128) and the
//                      MUSCL face-side states (Solver.cpp:69-121), fused; at stage 0 also the
//                      local time step (TimeStepCalculatorLocal.cpp:67-93).
//   face_flux_kernel   per face: Roe / slip-wall / freestream flux times area.
//   update_kernel      per cell: R = sum of +-flux*area in the reference's face order, then
//                      W(k) = W(n) - alpha_k dt/V R (SolverExplicit.cpp:326-378); the last stage
//                      also reduces the L2 / max norms of R.
#pragma once
#include "context.hpp"

namespace bes {

constexpr int kBlock = 256;

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ double warp_max(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
__device__ __forceinline__ double warp_min(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Batched conditions: blockIdx.y is the condition; its U, RS, FA, dt, dtmin, partials and
// freestream follow the first condition's at fixed strides ([condition][...]).  A condition
// whose Params::active entry is 0 is frozen: the sweeps skip it and the last update copies
// its state forward.
__device__ __forceinline__ bool condition_frozen(const Params& prm) {
  return prm.active != nullptr && prm.active[blockIdx.y] == 0;
}

// Cell sweep.  U is [5][nc]; RS is [5][ldr] with ldr >= nc*nslots + n_extra.  cfl_dev (may
// be null): a per-condition CFL number that replaces cfl (the implicit step's CFL control).
template <bool STAGE0, bool WRITE_GL>
__global__ void __launch_bounds__(kBlock) cell_recon_kernel(
    DevMesh m, Params prm, const double* __restrict__ U, double* __restrict__ RS, int64_t ldr,
    double* __restrict__ dt, double cfl, int local_dt, unsigned long long* __restrict__ dtmin,
    double* __restrict__ G_out, double* __restrict__ phi_out,
    const double* __restrict__ cfl_dev = nullptr) {
  const int nc = m.nc;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (condition_frozen(prm)) return;
  {
    const int64_t b = blockIdx.y;
    U += b * 5 * nc;
    RS += b * 5 * ldr;
    dt += b * nc;
    dtmin += b;
  }
  double dt_c = 1e300;
  if (c < nc) {
    double u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) u[v] = U[(int64_t)v * nc + c];
    int a[4];
    double ua[4][5];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a[k] = m.adj[k * nc + c];
      const int ak = a[k] >= 0 ? a[k] : c;
#pragma unroll
      for (int v = 0; v < 5; ++v) ua[k][v] = U[(int64_t)v * nc + ak];
    }
    const uint8_t flags = m.cflags[c];
    // ---- Green-Gauss gradient of the conserved variables
    double G[5][3];
#pragma unroll
    for (int v = 0; v < 5; ++v) G[v][0] = G[v][1] = G[v][2] = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double S[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) S[d] = m.Sc[(k * 3 + d) * nc + c];
      const double wk = a[k] >= 0 ? m.w[k * nc + c] : 1.0;
      const double wn = 1.0 - wk;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double fv = wk * u[v] + wn * ua[k][v];
#pragma unroll
        for (int d = 0; d < 3; ++d) G[v][d] = fma(S[d], fv, G[v][d]);
      }
      if (flags & (1u << k)) {
        // slip wall: momentum replaced by its tangential part (GradientGreenGauss.cpp:83-121)
        const int f = m.cface[k * nc + c];
        double n[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) n[d] = m.fn[(int64_t)d * m.nf + f];
        const double vn = u[1] * n[0] + u[2] * n[1] + u[3] * n[2];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const double t = u[1 + q] - vn * n[q];
#pragma unroll
          for (int d = 0; d < 3; ++d) G[1 + q][d] += (t * S[d] - u[1 + q] * S[d]);
        }
      }
    }
    const double iv = m.inv_vol[c];
#pragma unroll
    for (int v = 0; v < 5; ++v)
#pragma unroll
      for (int d = 0; d < 3; ++d) G[v][d] *= iv;
    // ---- Venkatakrishnan limiter; min over faces kept as a fraction (one division per var)
    double r[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d) r[k][d] = m.r[(k * 3 + d) * nc + c];
    const double eps2 = m.eps2[c];
    double phi[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      double dmin = u[v], dmax = u[v];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (a[k] >= 0) {
          dmin = ua[k][v] < dmin ? ua[k][v] : dmin;
          dmax = ua[k][v] > dmax ? ua[k][v] : dmax;
        }
      dmin -= u[v];
      dmax -= u[v];
      double bn = 1.0, bd = 1.0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (a[k] < 0) continue;
        const double d2 = 0.5 * (G[v][0] * r[k][0] + G[v][1] * r[k][1] + G[v][2] * r[k][2]);
        if (d2 == 0.0) continue;
        const double D1 = d2 > 0.0 ? dmax : dmin;
        const double num = D1 * D1 + eps2 + 2.0 * d2 * D1;
        const double den = D1 * D1 + 2.0 * d2 * d2 + D1 * d2 + eps2;
        if (num * bd < bn * den) {
          bn = num;
          bd = den;
        }
      }
      phi[v] = bn / bd;
    }
    // ---- MUSCL face-side states
    if (m.nslots == 1) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        double x = u[v];
#pragma unroll
        for (int d = 0; d < 3; ++d) x = fma(phi[v] * G[v][d], r[0][d], x);
        RS[(int64_t)v * ldr + c] = x;
      }
    } else {
#pragma unroll
      for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          double x = u[v];
#pragma unroll
          for (int d = 0; d < 3; ++d) x = fma(phi[v] * G[v][d], r[s][d], x);
          RS[(int64_t)v * ldr + (int64_t)s * nc + c] = x;
        }
    }
    if (flags & 0x10) {
      // reference lookup hitting another slot (quirk Q13): extra states after the main ones
      for (int k = 0; k < m.n_extra; ++k) {
        if (m.extra_cell[k] != c) continue;
        const int s = m.extra_m[k];
        for (int v = 0; v < 5; ++v) {
          double x = u[v];
          for (int d = 0; d < 3; ++d) x = fma(phi[v] * G[v][d], r[s][d], x);
          RS[(int64_t)v * ldr + (int64_t)nc * m.nslots + k] = x;
        }
      }
    }
    if (WRITE_GL) {
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        phi_out[(int64_t)v * nc + c] = phi[v];
#pragma unroll
        for (int d = 0; d < 3; ++d) G_out[(int64_t)(v * 3 + d) * nc + c] = G[v][d];
      }
    }
    if (STAGE0) {
      // local time step: CFL V / sum_d (c~ + |u_d|) L_d with c~ = sqrt(gamma) c (quirk Q3)
      const double ir = 1.0 / u[0];
      const double k2 = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
      const double e = u[4] - 0.5 * k2 * ir;
      const double p = prm.gas.gm1 * e;
      const double H = (u[4] + p) * ir;
      const double q2 = k2 * ir * ir;
      const double cs = sqrt(prm.gas.gamma * prm.gas.gm1 * (H - 0.5 * q2));
      double spec = 0.0;
#pragma unroll
      for (int d = 0; d < 3; ++d) spec += (cs + fabs(u[1 + d] * ir)) * m.plen[(int64_t)d * nc + c];
      dt_c = (cfl_dev ? cfl_dev[blockIdx.y] : cfl) * m.vol[c] / spec;
      dt[c] = dt_c;
    }
  }
  if (STAGE0 && !local_dt) {
    __shared__ double smin[kBlock / 32];
    double x = warp_min(dt_c);
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      x = threadIdx.x < kBlock / 32 ? smin[threadIdx.x] : 1e300;
      x = warp_min(x);
      // positive doubles order like their bit patterns
      if (threadIdx.x == 0) atomicMin(dtmin, (unsigned long long)__double_as_longlong(x));
    }
  }
}

template <bool WRITE_F>
__global__ void __launch_bounds__(kBlock) face_flux_kernel(
    DevMesh m, Params prm, const double* __restrict__ RS, int64_t ldr, double* __restrict__ FA,
    double* __restrict__ F_out, int* __restrict__ nan_flag) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int nf = m.nf;
  if (f >= nf || condition_frozen(prm)) return;
  const int64_t b = blockIdx.y;
  RS += b * 5 * ldr;
  FA += b * 5 * nf;
  const double* pinf = prm.pinf_dev + 6 * b;
  double UL[5], F[5];
  const int so = m.fsrc_own[f];
#pragma unroll
  for (int v = 0; v < 5; ++v) UL[v] = RS[(int64_t)v * ldr + so];
  double n[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) n[d] = m.fn[(int64_t)d * nf + f];
  if (f < m.nf_int) {
    double UR[5];
    const int sn = m.fsrc_nb[f];
#pragma unroll
    for (int v = 0; v < 5; ++v) UR[v] = RS[(int64_t)v * ldr + sn];
    roe_flux(prm.gas, UL, UR, n, F);
  } else if (f < m.nf_int + m.nf_slip) {
    slipwall_flux(prm.gas, UL, n, F);
  } else {
    freestream_flux(prm.gas, UL, pinf, n, F);
  }
  const double A = m.farea[f];
  bool bad = false;
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    FA[(int64_t)v * nf + f] = F[v] * A;
    if (WRITE_F) F_out[(int64_t)v * nf + f] = F[v];
    bad |= (F[v] != F[v]);
  }
  if (bad) atomicCAS(nan_flag, 0, f + 1);
}

template <bool LAST>
__global__ void __launch_bounds__(kBlock) update_kernel(
    DevMesh m, const double* __restrict__ FA, const double* __restrict__ Un,
    double* __restrict__ Uout, const double* __restrict__ dt,
    const unsigned long long* __restrict__ dtmin, int local_dt, double alpha,
    double* __restrict__ partials, double* __restrict__ R_out, const int32_t* active = nullptr) {
  const int nc = m.nc, nf = m.nf;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  {
    const int64_t b = blockIdx.y;
    FA += b * 5 * nf;
    Un += b * 5 * nc;
    Uout += b * 5 * nc;
    dt += b * nc;
    dtmin += b;
    partials += b * 10 * gridDim.x;
  }
  const bool frozen = active != nullptr && active[blockIdx.y] == 0;
  if (frozen && !LAST) return;
  double R[5] = {0, 0, 0, 0, 0};
  if (frozen) {
    // keep the state: the last stage's output becomes the next iteration's input
    if (c < nc)
#pragma unroll
      for (int v = 0; v < 5; ++v) Uout[(int64_t)v * nc + c] = Un[(int64_t)v * nc + c];
  } else if (c < nc) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int g = m.gface[q * nc + c];
      if (g == bes::kNoFace) continue;  // empty slot of a triangle
      const int f = g >= 0 ? g : ~g;
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        const double x = FA[(int64_t)v * nf + f];
        R[v] = g >= 0 ? R[v] + x : R[v] - x;
      }
    }
    const double dtc = local_dt ? dt[c] : __longlong_as_double((long long)*dtmin);
    const double coef = alpha * dtc * m.inv_vol[c];
#pragma unroll
    for (int v = 0; v < 5; ++v) Uout[(int64_t)v * nc + c] = Un[(int64_t)v * nc + c] - coef * R[v];
    if (R_out)
#pragma unroll
      for (int v = 0; v < 5; ++v) R_out[(int64_t)v * nc + c] = R[v];
  }
  if (LAST) {
    __shared__ double sh[10][kBlock / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double s = warp_sum(R[v] * R[v]);
      const double mx = warp_max(fabs(R[v]));
      if (lane == 0) {
        sh[v][wid] = s;
        sh[5 + v][wid] = mx;
      }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
      for (int k = 0; k < 10; ++k) {
        double x = lane < kBlock / 32 ? sh[k][lane] : 0.0;
        x = k < 5 ? warp_sum(x) : warp_max(x);
        if (lane == 0) partials[(int64_t)k * gridDim.x + blockIdx.x] = x;
      }
    }
  }
}

// One block per condition: reduce the per-block partials in a fixed order into
// history[iter][condition] (L2, max); iter = *iter_cur (set by freestream_step_kernel).
static __global__ void __launch_bounds__(kBlock) finalize_norms_kernel(
    const double* __restrict__ partials, int nblocks, double* __restrict__ hist,
    int64_t hist_cap, const int64_t* __restrict__ iter_cur) {
  __shared__ double sh[kBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t it = *iter_cur;
  const int nb = gridDim.x, b = blockIdx.x;
  partials += (int64_t)b * 10 * nblocks;
  for (int k = 0; k < 10; ++k) {
    double x = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
      const double y = partials[(int64_t)k * nblocks + b];
      x = k < 5 ? x + y : fmax(x, y);
    }
    x = k < 5 ? warp_sum(x) : warp_max(x);
    if (lane == 0) sh[wid] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      x = lane < kBlock / 32 ? sh[lane] : 0.0;
      x = k < 5 ? warp_sum(x) : warp_max(x);
      if (lane == 0 && it < hist_cap) hist[(it * nb + b) * 10 + k] = k < 5 ? sqrt(x) : x;
    }
    __syncthreads();
  }
}

static __global__ void reset_dtmin_kernel(unsigned long long* dtmin) {
  *dtmin = (unsigned long long)__double_as_longlong(1e300);
}

// State exchange: stage [nb][nc][5] in reference numbering <-> U [nb][5][nc] in the device
// numbering (new2ref: device cell -> reference cell).
static __global__ void state_from_stage_kernel(int nc, int nb, const int32_t* __restrict__ new2ref,
                                               const double* __restrict__ stage,
                                               double* __restrict__ U) {
  const int64_t n = (int64_t)nc * nb;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / nc, i = t - b * nc;
    const double* src = stage + (b * nc + new2ref[i]) * 5;
#pragma unroll
    for (int v = 0; v < 5; ++v) U[(b * 5 + v) * nc + i] = src[v];
  }
}
static __global__ void state_to_stage_kernel(int nc, int nb, const int32_t* __restrict__ new2ref,
                                             const double* __restrict__ U,
                                             double* __restrict__ stage) {
  const int64_t n = (int64_t)nc * nb;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / nc, i = t - b * nc;
    double* dst = stage + (b * nc + new2ref[i]) * 5;
#pragma unroll
    for (int v = 0; v < 5; ++v) dst[v] = U[(b * 5 + v) * nc + i];
  }
}

// First node of an explicit iteration (one block): every condition's freestream of this step
// and global-time-step reset, then the step counter and the history row.
static __global__ void freestream_step_kernel(Params prm, int nb, int64_t* step, double* pinf_dev,
                                              unsigned long long* dtmin, int64_t* iter_ctr,
                                              int64_t* iter_cur) {
  const int64_t st = *step;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    double p[6];
    freestream_from(prm.pinf0_dev + 6 * b, prm.ramp_steps, prm.ramp_frac, st, p);
    for (int i = 0; i < 6; ++i) pinf_dev[6 * b + i] = p[i];
    dtmin[b] = (unsigned long long)__double_as_longlong(1e300);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *step = st + 1;
    *iter_cur = *iter_ctr;
    *iter_ctr += 1;
  }
}

}  // namespace bes
