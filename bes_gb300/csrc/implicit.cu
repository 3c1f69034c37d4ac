// Implicit (backward-Euler) pseudo-time step on the GPU: SolverImplicit::timeStep_
// (src/SolverImplicit.cpp:293-345) with the AMGCL solve (src/CoefficientMatrix.cpp:210-325)
// replaced by right-preconditioned restarted GMRES with a block-Jacobi or colour-ordered
// block-ILU(0) preconditioner.  The system (Jacobian, preconditioner, Krylov vectors) is FP64
// for the plain method or FP32 for the defect correction; the residual, right-hand side,
// update and norms are always FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "context.hpp"
#include "implicit_kernels.cuh"

using namespace bes;

namespace {

#define IMP_TRY(ctx, call)                                                       \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      (ctx)->last_error = std::string(#call) + ": " + cudaGetErrorString(e_);    \
      return BES_ERR_CUDA;                                                       \
    }                                                                            \
  } while (0)

inline int nblk(int64_t n, int b) { return (int)((n + b - 1) / b); }

int imp_malloc(bes_ctx* c, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 8);
  if (e != cudaSuccess) {
    c->last_error = std::string("cudaMalloc (implicit): ") + cudaGetErrorString(e);
    return BES_ERR_CUDA;
  }
  c->allocations.push_back(*p);
  return BES_OK;
}

inline int64_t basis_stride(int64_t nc) { return (5 * nc + 63) / 64 * 64; }

template <class T>
struct Sys {
  bes_ctx* c;
  int nc;
  int64_t N;
  T* A;
  T* LU;
  T* Dinv;
  T* Dc;
  T* b;
  T* V;
  T* Z;
  T* W;
  T* X;
  bool packed;  // precision 2: the Krylov products and sweeps read the 16-bit copies
  const __half2 *A16, *LU16, *D16;
  const float *As, *LUs, *Ds;
  bool basis16;  // precision 2: FP16 Krylov basis; the preconditioner reads Vx
  T* Vx;         // FP32 copy of the newest basis vector (basis16 only)
  cudaStream_t s;
  explicit Sys(bes_ctx* ctx) : c(ctx) {
    ImplicitBuffers& I = ctx->imp;
    nc = ctx->soa.nc;
    N = 5LL * nc;
    ldv = basis_stride(nc);
    A = (T*)I.A;
    LU = (T*)I.LU;
    Dinv = (T*)I.Dinv;
    Dc = (T*)I.Dc;
    b = (T*)I.b;
    V = (T*)I.V;
    Z = (T*)I.Z;
    W = (T*)I.W;
    X = (T*)I.X;
    packed = I.packed;
    A16 = (const __half2*)I.A16;
    LU16 = (const __half2*)I.LU16;
    D16 = (const __half2*)I.D16;
    As = I.As;
    LUs = I.LUs;
    Ds = I.Ds;
    basis16 = I.basis16;
    Vx = (T*)I.Vx;
    s = ctx->stream;
  }
  int64_t ldv;  // stride of the Krylov basis: N rounded up to 64 elements (16-byte loads)
  T* Vk(int k) const { return V + (int64_t)k * ldv; }
};

// reduce rows of c->imp.red and copy them to the host
int reduce_to_host(bes_ctx* c, int nrows, int nblocks, int nsum, int sqrt_sums, double* host) {
  reduce_rows_kernel<<<nrows, 256, 0, c->stream>>>(c->imp.red, nblocks, nsum, sqrt_sums,
                                                   c->imp.red_out);
  ++c->launches;
  IMP_TRY(c, cudaMemcpyAsync(host, c->imp.red_out, nrows * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream));
  IMP_TRY(c, cudaStreamSynchronize(c->stream));
  return BES_OK;
}

// 16-bit block-scaled copies (precision 2; T is float there)
template <class T>
void enqueue_pack(const Sys<T>& S, const T* src, int slot0, int nslots, void* H, float* sc) {
  if constexpr (std::is_same<T, float>::value) {
    pack_blocks_kernel<<<dim3(nblk(S.nc, 256), nslots), 256, 0, S.s>>>(src, slot0, S.nc,
                                                                       (__half2*)H, sc);
    ++S.c->launches;
  }
}

// y = A x, or y = b - A x when b is given
template <class T>
void spmv(const Sys<T>& S, const T* x, const T* b, T* y) {
  if constexpr (std::is_same<T, float>::value) {
    if (S.packed) {
      spmv_packed_kernel<<<nblk(S.nc, 256), 256, 0, S.s>>>(S.c->dm, S.A16, S.As, x, b, y);
      ++S.c->launches;
      return;
    }
  }
  spmv_kernel<T><<<nblk(S.nc, 256), 256, 0, S.s>>>(S.c->dm, S.A, x, b, y);
  ++S.c->launches;
}

inline bool uses_ilu(const bes_ctx* c) { return c->opt.linear_solver == 1 || c->opt.linear_solver == 2; }

// Enqueue the block-ILU(0) sweeps in place on S.Z (stage by stage), for graph capture.
template <class T>
void enqueue_ilu_sweeps(const Sys<T>& S) {
  bes_ctx* c = S.c;
  const SoaMesh& M = c->soa;
  for (int k = 0; k < M.n_stages; ++k) {
    const int n = M.stage_off[k + 1] - M.stage_off[k];
    ilu_lower_kernel<T><<<nblk(n, 128), 128, 0, S.s>>>(c->dm, c->imp.stage_rows + M.stage_off[k],
                                                       n, c->imp.ilu_pos, S.LU, S.Z, S.Z);
  }
  for (int k = M.n_stages - 1; k >= 0; --k) {
    const int n = M.stage_off[k + 1] - M.stage_off[k];
    ilu_upper_kernel<T><<<nblk(n, 128), 128, 0, S.s>>>(c->dm, c->imp.stage_rows + M.stage_off[k],
                                                       n, c->imp.ilu_pos, S.LU, S.Dinv, S.Z);
  }
}

template <class T>
void enqueue_ilu_factor(const Sys<T>& S) {
  bes_ctx* c = S.c;
  const SoaMesh& M = c->soa;
  // the factors overwrite a copy: the Krylov products need the unfactored matrix
  cudaMemcpyAsync(S.LU, S.A, (size_t)125 * S.nc * sizeof(T), cudaMemcpyDeviceToDevice, S.s);
  // per stage: the factorisation of its rows, then the inverses of their diagonal blocks (a
  // separate kernel keeps the factorisation's registers free of the 5x10 elimination array)
  for (int k = 0; k < M.n_stages; ++k) {
    const int n = M.stage_off[k + 1] - M.stage_off[k];
    if (c->imp.use_colour_ranges) {
      ilu_factor_kernel<T, true><<<nblk(n, 128), 128, 0, S.s>>>(c->dm, nullptr, n, nullptr, S.LU,
                                                                S.Dinv, M.stage_off[k]);
      ilu_invert_kernel<T, true><<<nblk(n, 128), 128, 0, S.s>>>(c->dm, nullptr, n, S.LU, S.Dinv,
                                                                M.stage_off[k]);
    } else {
      ilu_factor_kernel<T><<<nblk(n, 128), 128, 0, S.s>>>(c->dm, c->imp.stage_rows + M.stage_off[k],
                                                          n, c->imp.ilu_pos, S.LU, S.Dinv);
      ilu_invert_kernel<T><<<nblk(n, 128), 128, 0, S.s>>>(c->dm, c->imp.stage_rows + M.stage_off[k],
                                                          n, S.LU, S.Dinv);
    }
  }
  if (S.packed) {
    enqueue_pack(S, S.LU, 1, 4, c->imp.LU16, c->imp.LUs);
    enqueue_pack(S, S.Dinv, 0, 1, c->imp.D16, c->imp.Ds);
  }
}

// Colour-range sweeps (ilu_colour_kernel) from `in` into S.Z: colours 1..C-2 forward, the last
// colour's two solves fused, colours C-2..0 backward.
template <class T>
void enqueue_ilu_colour_sweeps(const Sys<T>& S, const T* in) {
  bes_ctx* c = S.c;
  const SoaMesh& M = c->soa;
  const int C = M.n_stages;
  const int s1 = M.stage_off[1];
  auto range = [&](int k, int& r0, int& r1) { r0 = M.stage_off[k]; r1 = M.stage_off[k + 1]; };
  int r0, r1;
  if constexpr (std::is_same<T, float>::value) {
    if (S.packed) {
      for (int k = 1; k < C - 1; ++k) {
        range(k, r0, r1);
        ilu_colour_packed_kernel<true, false><<<nblk(r1 - r0, 128), 128, 0, S.s>>>(
            c->dm, r0, r1, s1, S.LU16, S.LUs, S.D16, S.Ds, in, S.Z);
      }
      range(C - 1, r0, r1);
      ilu_colour_packed_kernel<true, true><<<nblk(r1 - r0, 128), 128, 0, S.s>>>(
          c->dm, r0, r1, s1, S.LU16, S.LUs, S.D16, S.Ds, in, S.Z);
      for (int k = C - 2; k >= 0; --k) {
        range(k, r0, r1);
        ilu_colour_packed_kernel<false, true><<<nblk(r1 - r0, 128), 128, 0, S.s>>>(
            c->dm, r0, r1, s1, S.LU16, S.LUs, S.D16, S.Ds, in, S.Z);
      }
      return;
    }
  }
  for (int k = 1; k < C - 1; ++k) {
    range(k, r0, r1);
    ilu_colour_kernel<T, true, false><<<nblk(r1 - r0, 128), 128, 0, S.s>>>(
        c->dm, r0, r1, s1, S.LU, S.Dinv, in, S.Z);
  }
  range(C - 1, r0, r1);
  ilu_colour_kernel<T, true, true><<<nblk(r1 - r0, 128), 128, 0, S.s>>>(c->dm, r0, r1, s1, S.LU,
                                                                       S.Dinv, in, S.Z);
  for (int k = C - 2; k >= 0; --k) {
    range(k, r0, r1);
    ilu_colour_kernel<T, false, true><<<nblk(r1 - r0, 128), 128, 0, S.s>>>(
        c->dm, r0, r1, s1, S.LU, S.Dinv, in, S.Z);
  }
}

// True when the factorisation order is the identity and every stage is a contiguous range of
// cells in increasing order (colour order on the colour-major numbering).
inline bool colour_ranges(const SoaMesh& M) {
  if (M.n_stages < 1) return false;
  for (int64_t i = 0; i < (int64_t)M.ilu_pos.size(); ++i)
    if (M.ilu_pos[i] != i || M.stage_rows[i] != i) return false;
  return true;
}

// Capture the stage-by-stage ILU work once per context as CUDA graphs (hundreds of small
// kernels under level scheduling).  With colour ranges there is one sweep graph per input
// vector (the Krylov vectors V_0..V_m and W), so that no copy of the input is needed.
template <class T>
int ensure_ilu_graphs(const Sys<T>& S) {
  bes_ctx* c = S.c;
  if (c->imp.apply_graph || !c->imp.colour_graphs.empty()) return BES_OK;
  cudaGraph_t g;
  IMP_TRY(c, cudaStreamBeginCapture(S.s, cudaStreamCaptureModeThreadLocal));
  enqueue_ilu_factor(S);
  IMP_TRY(c, cudaStreamEndCapture(S.s, &g));
  IMP_TRY(c, cudaGraphInstantiate(&c->imp.factor_graph, g, 0));
  cudaGraphDestroy(g);
  if (c->imp.use_colour_ranges) {
    // inputs V_0..V_m, then W; with an FP16 basis the FP32 copy Vx, then W
    const int nin = S.basis16 ? 2 : c->opt.gmres_restart + 2;
    for (int q = 0; q < nin; ++q) {
      const T* in = q + 1 < nin ? (S.basis16 ? S.Vx : S.Vk(q)) : S.W;
      IMP_TRY(c, cudaStreamBeginCapture(S.s, cudaStreamCaptureModeThreadLocal));
      enqueue_ilu_colour_sweeps(S, in);
      IMP_TRY(c, cudaStreamEndCapture(S.s, &g));
      cudaGraphExec_t ge = nullptr;
      IMP_TRY(c, cudaGraphInstantiate(&ge, g, 0));
      cudaGraphDestroy(g);
      c->imp.colour_graphs.push_back(ge);
    }
    return BES_OK;
  }
  IMP_TRY(c, cudaStreamBeginCapture(S.s, cudaStreamCaptureModeThreadLocal));
  enqueue_ilu_sweeps(S);
  IMP_TRY(c, cudaStreamEndCapture(S.s, &g));
  IMP_TRY(c, cudaGraphInstantiate(&c->imp.apply_graph, g, 0));
  cudaGraphDestroy(g);
  return BES_OK;
}

// out = M^{-1} in (out is always S.Z)
template <class T>
void precond_apply(const Sys<T>& S, const T* in, T* out) {
  bes_ctx* c = S.c;
  if (uses_ilu(c) && c->imp.use_colour_ranges) {
    // out is S.Z; in is one of V_0..V_m (graph q = its index) or Vx (graph 0), or W (the
    // last graph)
    const int64_t q = in == S.W ? (int64_t)c->imp.colour_graphs.size() - 1
                                : (S.basis16 ? 0 : (in - S.V) / S.ldv);
    cudaGraphLaunch(c->imp.colour_graphs[q], S.s);
    c->launches += 2 * c->soa.n_stages - 1;
  } else if (uses_ilu(c)) {
    if (in != out)
      cudaMemcpyAsync(out, in, (size_t)S.N * sizeof(T), cudaMemcpyDeviceToDevice, S.s);
    cudaGraphLaunch(c->imp.apply_graph, S.s);
    c->launches += 2 * c->soa.n_stages;
  } else {
    if constexpr (std::is_same<T, float>::value) {
      if (S.packed) {
        jacobi_apply_packed_kernel<<<nblk(S.nc, 256), 256, 0, S.s>>>(S.nc, S.D16, S.Ds, in, out);
        ++S.c->launches;
        return;
      }
    }
    jacobi_apply_kernel<T><<<nblk(S.nc, 256), 256, 0, S.s>>>(S.nc, S.Dinv, in, out);
    ++S.c->launches;
  }
}

template <class T>
int precond_setup(const Sys<T>& S) {
  bes_ctx* c = S.c;
  if (!uses_ilu(c)) return BES_OK;  // block Jacobi inverted during assembly
  int rc = ensure_ilu_graphs(S);
  if (rc) return rc;
  prof_begin(c, PROF_ILU_FACTOR);
  IMP_TRY(c, cudaGraphLaunch(c->imp.factor_graph, S.s));
  prof_end(c, PROF_ILU_FACTOR);
  c->launches += 2 * c->soa.n_stages + (S.packed ? 2 : 0);
  return BES_OK;
}

// Residual, first-order Jacobians and the assembled system at the current state; returns the
// FP64 norms: L2[5] and max[5] of the Dt/V-scaled right-hand side, L2[5] of the residual R.
template <class T>
int assemble(bes_ctx* c, double cfl, double* norms15) {
  Sys<T> S(c);
  const DevMesh& m = c->dm;
  const bes_options& o = c->opt;
  const int local = o.local_time_step;
  double* U = c->U[c->cur];
  prof_begin(c, PROF_RESIDUAL);
  reset_dtmin_kernel<<<1, 1, 0, S.s>>>(c->dtmin);
  ++S.c->launches;
  cell_recon_kernel<true, false><<<nblk(m.nc, kBlock), kBlock, 0, S.s>>>(
      m, c->prm, U, c->RS, c->rs_ld, c->dt, cfl, local, c->dtmin, nullptr, nullptr);
  ++S.c->launches;
  face_flux_kernel<false><<<nblk(m.nf, kBlock), kBlock, 0, S.s>>>(m, c->prm, c->RS, c->rs_ld,
                                                                  c->FA, nullptr, c->nan_flag);
  ++S.c->launches;
  prof_end(c, PROF_RESIDUAL);
  FaceLocal fl{c->imp.m_own, c->imp.m_nb};
  prof_begin(c, PROF_JACOBIAN);
  face_jacobian_kernel<T><<<nblk(m.nf, 128), 128, 0, S.s>>>(
      m, c->prm, fl, U, c->dt, c->dtmin, local, o.jacobian_repeat, S.A, S.Dc);
  ++S.c->launches;
  prof_end(c, PROF_JACOBIAN);
  const int nb = nblk(m.nc, 128);
  prof_begin(c, PROF_ASSEMBLE);
  cell_assemble_kernel<T><<<nb, 128, 0, S.s>>>(m, c->FA, c->dt, c->dtmin, local,
                                               o.jacobian_repeat, S.Dc, S.A,
                                               uses_ilu(c) ? nullptr : S.Dinv,
                                               c->imp.rhs, S.b, c->imp.red);
  ++S.c->launches;
  if (S.packed) {
    enqueue_pack(S, S.A, 0, 5, c->imp.A16, c->imp.As);
    if (!uses_ilu(c)) enqueue_pack(S, S.Dinv, 0, 1, c->imp.D16, c->imp.Ds);
  }
  prof_end(c, PROF_ASSEMBLE);
  IMP_TRY(c, cudaGetLastError());
  double r[15];
  const int rc = reduce_to_host(c, 15, nb, 10, 1, r);
  prof_collect(c);
  // norms15: L2 of the right-hand side [5], max of the right-hand side [5], L2 of R [5]
  for (int v = 0; v < 5; ++v) {
    norms15[v] = r[v];
    norms15[5 + v] = r[10 + v];
    norms15[10 + v] = r[5 + v];
  }
  return rc;
}

// Right-preconditioned GMRES(m), x0 = 0, classical Gram-Schmidt with a conditional second
// pass, Givens rotations; stops when |g_{j+1}| <= tol |b| (AMGCL gmres.hpp:163,214 semantics).
template <class T, class B>
int gmres_basis(bes_ctx* c, int& iters_out, double& rel_out) {
  Sys<T> S(c);
  constexpr bool kBasis16 = !std::is_same<T, B>::value;
  B* const Vb = (B*)c->imp.V;
  auto Vk = [&](int k) { return Vb + (int64_t)k * S.ldv; };
  // the preconditioner's input: the basis vector itself, or its FP32 copy
  auto pin = [&](int k) -> const T* {
    if constexpr (kBasis16) return S.Vx;
    else return Vk(k);
  };
  const bes_options& o = c->opt;
  const int mr = o.gmres_restart;
  const int maxiter = o.linear_solver_max_iter;
  const double tol = o.linear_solver_tol;
  const int G = kRedBlocks;
  double* red = c->imp.red;
  zero_kernel<T><<<G, 256, 0, S.s>>>(S.X, S.N);
  ++S.c->launches;
  norm2_kernel<T><<<G, 256, 0, S.s>>>(S.b, S.N, red);
  ++S.c->launches;
  double norm_b2;
  int rc = reduce_to_host(c, 1, G, 1, 0, &norm_b2);
  if (rc) return rc;
  const double norm_b = std::sqrt(norm_b2);
  iters_out = 0;
  rel_out = 0.0;
  if (norm_b == 0.0) return BES_OK;
  const double eps = tol * norm_b;
  std::vector<double> H((mr + 1) * mr, 0.0), cs(mr), sn(mr), g(mr + 1), y(mr);
  int iter = 0;
  double norm_r = norm_b;
  scale_kernel<T><<<G, 256, 0, S.s>>>(S.W, S.b, 1.0, S.N);  // r = b
  double beta = norm_b;
  ++S.c->launches;
  while (true) {
    if (beta < eps || iter >= maxiter) break;
    if constexpr (kBasis16)
      basis_start_kernel<<<G, 256, 0, S.s>>>(Vk(0), S.Vx, S.W, 1.0 / beta, S.N);
    else
      scale_kernel<T><<<G, 256, 0, S.s>>>(Vk(0), S.W, 1.0 / beta, S.N);
    ++S.c->launches;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    while (j < mr && iter < maxiter) {
      prof_begin(c, PROF_PRECOND);
      precond_apply(S, pin(j), S.Z);
      prof_end(c, PROF_PRECOND);
      prof_begin(c, PROF_SPMV);
      spmv<T>(S, S.Z, nullptr, S.W);
      prof_end(c, PROF_SPMV);
      // classical Gram-Schmidt with a conditional second pass (gs_* kernels); the
      // coefficients stay on the device and reach the host once per iteration
      double* dev = c->imp.red_out;
      const int nv = j + 1;
      prof_begin(c, PROF_ORTHO);
      T* const vx = kBasis16 ? S.Vx : nullptr;
      launch_gs_dots<T, B>(nv, G, S.s, Vb, S.ldv, S.W, S.N, red);
      reduce_rows_kernel<<<nv + 1, 256, 0, S.s>>>(red, G, nv + 1, 0, dev);
      float* devf = c->imp.red_out_f;
      gs_decide_kernel<<<1, 64, 0, S.s>>>(dev, devf, nv, 1);
      launch_gs_update<T, B, GS_FINAL1>(nv, G, S.s, Vk(j + 1), vx, S.W, Vb, S.ldv, dev, devf,
                                        S.N, red);
      launch_gs_update<T, B, GS_REORTH>(nv, G, S.s, nullptr, nullptr, S.W, Vb, S.ldv, dev, devf,
                                        S.N, red);
      reduce_rows_kernel<<<nv + 1, 256, 0, S.s>>>(red, G, nv + 1, 0, dev + kGsH2);
      gs_decide_kernel<<<1, 64, 0, S.s>>>(dev, devf, nv, 2);
      launch_gs_update<T, B, GS_FINAL2>(nv, G, S.s, Vk(j + 1), vx, S.W, Vb, S.ldv, dev, devf,
                                        S.N, red);
      prof_end(c, PROF_ORTHO);
      S.c->launches += 8;
      double hbuf[kGsScalars];
      IMP_TRY(c, cudaMemcpyAsync(hbuf, dev, sizeof(hbuf), cudaMemcpyDeviceToHost, S.s));
      IMP_TRY(c, cudaStreamSynchronize(S.s));
      prof_collect(c);
      const bool second = hbuf[kGsFlag] != 0.0;
      if (second) ++c->imp.gs_second_passes;
      for (int i = 0; i <= j; ++i) H[i * mr + j] = hbuf[i] + (second ? hbuf[kGsH2 + i] : 0.0);
      H[(j + 1) * mr + j] = hbuf[kGsNorm];
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * H[i * mr + j] + sn[i] * H[(i + 1) * mr + j];
        H[(i + 1) * mr + j] = -sn[i] * H[i * mr + j] + cs[i] * H[(i + 1) * mr + j];
        H[i * mr + j] = t;
      }
      const double a = H[j * mr + j], cc = H[(j + 1) * mr + j];
      const double d = std::sqrt(a * a + cc * cc);
      cs[j] = (d == 0.0) ? 1.0 : a / d;
      sn[j] = (d == 0.0) ? 0.0 : cc / d;
      H[j * mr + j] = d;
      H[(j + 1) * mr + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      ++j;
      ++iter;
      if (std::fabs(g[j]) <= eps) break;
    }
    for (int i = j - 1; i >= 0; --i) {
      double s = g[i];
      for (int k = i + 1; k < j; ++k) s -= H[i * mr + k] * y[k];
      y[i] = s / H[i * mr + i];
    }
    IMP_TRY(c, cudaMemcpyAsync(c->imp.coef, y.data(), j * sizeof(double), cudaMemcpyHostToDevice, S.s));
    lincomb_kernel<T, B><<<G, 256, 0, S.s>>>(S.W, Vb, S.ldv, j, c->imp.coef, S.N);
    ++S.c->launches;
    precond_apply(S, S.W, S.Z);
    add_kernel<T><<<G, 256, 0, S.s>>>(S.X, S.Z, S.N);
    ++S.c->launches;
    spmv<T>(S, S.X, S.b, S.W);  // r = b - A x
    norm2_kernel<T><<<G, 256, 0, S.s>>>(S.W, S.N, red);
    ++S.c->launches;
    double nr2;
    if ((rc = reduce_to_host(c, 1, G, 1, 0, &nr2))) return rc;
    norm_r = std::sqrt(nr2);
    if (norm_r <= eps || iter >= maxiter) break;
    beta = norm_r;
  }
  iters_out = iter;
  rel_out = norm_r / norm_b;
  IMP_TRY(c, cudaGetLastError());
  return BES_OK;
}

template <class T>
int gmres(bes_ctx* c, int& iters_out, double& rel_out) {
  if constexpr (std::is_same<T, float>::value)
    if (c->imp.basis16) return gmres_basis<float, __half>(c, iters_out, rel_out);
  return gmres_basis<T, T>(c, iters_out, rel_out);
}

double cfl_for_step(const bes_ctx* c) {
  const bes_options& o = c->opt;
  if (o.cfl_ramp_steps > 0) {
    const int64_t k = c->imp.step_count;
    if (k >= o.cfl_ramp_steps - 1 || o.cfl_ramp_steps == 1) return o.cfl_ramp_end;
    const double t = (double)k / (double)(o.cfl_ramp_steps - 1);
    return o.cfl_ramp_start * std::pow(o.cfl_ramp_end / o.cfl_ramp_start, t);
  }
  return c->imp.cfl_actual;
}

template <class T>
int implicit_step(bes_ctx* c, double* hist) {
  ImplicitBuffers& I = c->imp;
  const bes_options& o = c->opt;
  for (int v = 0; v < 5; ++v) I.maxres_old[v] = I.maxres[v];
  const double cfl = cfl_for_step(c);
  double P[6];
  freestream_at(c->prm, c->host_step, P);  // FREESTREAM_RAMP
  IMP_TRY(c, cudaMemcpyAsync(c->pinf_dev, P, sizeof(P), cudaMemcpyHostToDevice, c->stream));
  double norms[15];
  int rc = assemble<T>(c, cfl, norms);
  if (rc) return rc;
  rc = check_nan_public(c);
  if (rc) return rc;
  Sys<T> S(c);
  rc = precond_setup(S);
  if (rc) return rc;
  int iters = 0;
  double rel = 0.0;
  rc = gmres<T>(c, iters, rel);
  if (rc) return rc;
  prof_begin(c, PROF_OTHER);
  state_update_kernel<T><<<kRedBlocks, 256, 0, c->stream>>>(c->U[c->cur], S.X, (int64_t)S.nc);
  prof_end(c, PROF_OTHER);
  ++c->launches;
  IMP_TRY(c, cudaGetLastError());
  for (int v = 0; v < 5; ++v) I.maxres[v] = norms[5 + v];
  if (o.cfl_ramp_steps <= 0 && o.adaptive_courant_num_max > o.courant_num) {
    // SolverImplicit::adaptCourantNum_ (src/SolverImplicit.cpp:530-550)
    const int idx = (I.maxres_old[0] > I.maxres[0]) ? 1 : 0;
    I.cfl_actual *= std::pow(I.maxres_old[0] / I.maxres[0], o.adaptive_courant_num_exponent[idx]);
    I.cfl_actual = std::max(o.courant_num, I.cfl_actual);
    I.cfl_actual = std::min(o.adaptive_courant_num_max, I.cfl_actual);
  }
  I.last_iters = iters;
  I.total_lin_iters += iters;
  I.last_err = rel;
  if (hist) {
    for (int k = 0; k < 10; ++k) hist[k] = norms[k];
    hist[10] = cfl;
    hist[11] = I.cfl_actual;
    hist[12] = iters;
    hist[13] = rel;
    for (int k = 0; k < 5; ++k) hist[14 + k] = norms[10 + k];
  }
  ++I.step_count;
  ++c->host_step;
  return BES_OK;
}

// A batched context's condition b seen as a single-condition context: its state, face
// states, fluxes, time steps and freestream, and its CFL controller, swapped in for the
// duration of one implicit step (the implicit buffers are shared by all conditions).
struct ConditionView {
  bes_ctx* c;
  double* U[2];
  double *RS, *FA, *dt, *pinf;
  unsigned long long* dtmin;
  Params prm;
  bes_ctx::CondImplicit saved;
  int nb;
  ConditionView(bes_ctx* ctx, int b) : c(ctx) {
    const int64_t nc = c->soa.nc, nf = c->soa.nf;
    for (int k = 0; k < 2; ++k) U[k] = c->U[k];
    RS = c->RS; FA = c->FA; dt = c->dt; pinf = c->pinf_dev; dtmin = c->dtmin;
    prm = c->prm;
    nb = c->nb;
    for (int k = 0; k < 2; ++k) c->U[k] += (int64_t)b * 5 * nc;
    c->RS += (int64_t)b * 5 * c->rs_ld;
    c->FA += (int64_t)b * 5 * nf;
    c->dt += (int64_t)b * nc;
    c->dtmin += b;
    c->pinf_dev += 6 * b;
    c->prm.pinf_dev = c->pinf_dev;
    c->prm.active = nullptr;
    for (int i = 0; i < 6; ++i) c->prm.pinf[i] = c->pinf0_host[6 * b + i];
    c->nb = 1;
    swap_scalars(c->cond_imp[b]);
  }
  void swap_scalars(bes_ctx::CondImplicit& s) {
    ImplicitBuffers& I = c->imp;
    std::swap(s.cfl_actual, I.cfl_actual);
    for (int v = 0; v < 5; ++v) {
      std::swap(s.maxres[v], I.maxres[v]);
      std::swap(s.maxres_old[v], I.maxres_old[v]);
    }
    std::swap(s.step_count, I.step_count);
    std::swap(s.host_step, c->host_step);
  }
  void release(int b) {
    swap_scalars(c->cond_imp[b]);
    for (int k = 0; k < 2; ++k) c->U[k] = U[k];
    c->RS = RS; c->FA = FA; c->dt = dt; c->pinf_dev = pinf; c->dtmin = dtmin;
    c->prm = prm;
    c->nb = nb;
  }
};

// n implicit steps of every condition of a batch, condition after condition within a step;
// history [n][nb][19]
int implicit_steps_batch(bes_ctx* ctx, int64_t n, double* history) {
  const int nb = ctx->nb;
  for (int64_t i = 0; i < n; ++i) {
    for (int b = 0; b < nb; ++b) {
      ConditionView view(ctx, b);
      double* h = history ? history + (i * nb + b) * 19 : nullptr;
      const int rc = ctx->imp.prec ? implicit_step<float>(ctx, h) : implicit_step<double>(ctx, h);
      view.release(b);
      if (rc) return rc;
    }
    ++ctx->imp.step_count;
    ++ctx->host_step;
  }
  IMP_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  prof_collect(ctx);
  return BES_OK;
}

}  // namespace

namespace bes {

void prof_begin(bes_ctx* c, int cat) {
  Profiler& P = c->prof;
  if (!P.on) return;
  if (P.next * 2 + 2 > (int)P.pool.size()) {
    for (int q = 0; q < 64; ++q) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      P.pool.push_back(e);
    }
  }
  const int pr = P.next++;
  P.open_pair[cat] = pr;
  cudaEventRecord(P.pool[2 * pr], c->stream);
}

void prof_end(bes_ctx* c, int cat) {
  Profiler& P = c->prof;
  if (!P.on) return;
  const int pr = P.open_pair[cat];
  cudaEventRecord(P.pool[2 * pr + 1], c->stream);
  P.pending.push_back({cat, pr});
}

void prof_collect(bes_ctx* c) {
  Profiler& P = c->prof;
  if (!P.on) return;
  cudaStreamSynchronize(c->stream);
  for (auto& q : P.pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, P.pool[2 * q.second], P.pool[2 * q.second + 1]) == cudaSuccess) {
      P.ms[q.first] += ms;
      P.count[q.first] += 1;
    }
  }
  P.pending.clear();
  P.next = 0;
}

int implicit_allocate(bes_ctx* c) {
  ImplicitBuffers& I = c->imp;
  const bes_options& o = c->opt;
  if (o.gmres_restart < 1 || o.gmres_restart > 32) {
    c->last_error = "GMRES_RESTART must be between 1 and 32";
    return BES_ERR_UNSUPPORTED;
  }
  if (o.precision < 0 || o.precision > 2) {
    c->last_error = "precision must be 0 (FP64 system), 1 (FP32 system) or 2 (FP32 system, "
                    "16-bit block-scaled matrix storage)";
    return BES_ERR_UNSUPPORTED;
  }
  I.prec = o.precision ? 1 : 0;
  I.packed = o.precision == 2;
  I.tsize = I.prec ? sizeof(float) : sizeof(double);
  const SoaMesh& M = c->soa;
  const int64_t nc = M.nc, nf = M.nf, N = 5 * nc;
  int rc = 0;
  rc |= imp_malloc(c, &I.A, 125 * nc * I.tsize);
  rc |= imp_malloc(c, &I.Dinv, 25 * nc * I.tsize);
  if (o.linear_solver < 0 || o.linear_solver > 2) {
    c->last_error = "linear_solver must be 0 (block Jacobi), 1 (block ILU(0), colour order) or 2 "
                    "(block ILU(0), RCM order, level scheduled)";
    return BES_ERR_UNSUPPORTED;
  }
  if (o.linear_solver == 2) build_ilu_schedule(c->soa, true);
  I.use_colour_ranges = o.linear_solver == 1 && colour_ranges(c->soa);
  if (I.packed && uses_ilu(c) && !I.use_colour_ranges) {
    c->last_error = "precision 2 runs block Jacobi or the colour-ordered block ILU(0)";
    return BES_ERR_UNSUPPORTED;
  }
  if (uses_ilu(c)) rc |= imp_malloc(c, &I.LU, 125 * nc * I.tsize);
  if (I.packed) {
    rc |= imp_malloc(c, &I.A16, 5 * 13 * nc * sizeof(__half2));
    rc |= imp_malloc(c, (void**)&I.As, 5 * nc * sizeof(float));
    rc |= imp_malloc(c, &I.D16, 13 * nc * sizeof(__half2));
    rc |= imp_malloc(c, (void**)&I.Ds, nc * sizeof(float));
    if (uses_ilu(c)) {
      rc |= imp_malloc(c, &I.LU16, 4 * 13 * nc * sizeof(__half2));
      rc |= imp_malloc(c, (void**)&I.LUs, 4 * nc * sizeof(float));
    }
  }
  rc |= imp_malloc(c, &I.Dc, 50 * nf * I.tsize);
  rc |= imp_malloc(c, &I.b, N * I.tsize);
  I.basis16 = I.packed;
  rc |= imp_malloc(c, &I.V, (size_t)(o.gmres_restart + 1) * basis_stride(nc) *
                                (I.basis16 ? sizeof(__half) : I.tsize));
  if (I.basis16) rc |= imp_malloc(c, &I.Vx, N * sizeof(float));
  rc |= imp_malloc(c, &I.Z, N * I.tsize);
  rc |= imp_malloc(c, &I.W, N * I.tsize);
  rc |= imp_malloc(c, &I.X, N * I.tsize);
  rc |= imp_malloc(c, (void**)&I.rhs, N * sizeof(double));
  rc |= imp_malloc(c, (void**)&I.red, 64 * (size_t)std::max<int64_t>(kRedBlocks, nblk(nc, 128)) * sizeof(double));
  rc |= imp_malloc(c, (void**)&I.red_out, 128 * sizeof(double));
  rc |= imp_malloc(c, (void**)&I.red_out_f, 128 * sizeof(float));
  rc |= imp_malloc(c, (void**)&I.coef, 64 * sizeof(double));
  rc |= imp_malloc(c, (void**)&I.m_own, nf);
  rc |= imp_malloc(c, (void**)&I.m_nb, nf);
  rc |= imp_malloc(c, (void**)&I.stage_rows, nc * sizeof(int32_t));
  rc |= imp_malloc(c, (void**)&I.ilu_pos, nc * sizeof(int32_t));
  if (rc) return BES_ERR_CUDA;
  IMP_TRY(c, cudaMemset(I.A, 0, 125 * nc * I.tsize));  // empty slots stay zero
  IMP_TRY(c, cudaMemcpy(I.m_own, M.f_m_own.data(), nf, cudaMemcpyHostToDevice));
  IMP_TRY(c, cudaMemcpy(I.m_nb, M.f_m_nb.data(), nf, cudaMemcpyHostToDevice));
  IMP_TRY(c, cudaMemcpy(I.stage_rows, M.stage_rows.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice));
  IMP_TRY(c, cudaMemcpy(I.ilu_pos, M.ilu_pos.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice));
  I.cfl_actual = o.courant_num;
  return BES_OK;
}

}  // namespace bes

extern "C" {

int bes_implicit_steps(bes_ctx* ctx, int64_t n, double* history) {
  if (!ctx || n < 0) return BES_ERR_INVALID;
  if (ctx->opt.solver_type != 1 || !ctx->imp.A) {
    ctx->last_error = "context was not created for the implicit solver";
    return BES_ERR_INVALID;
  }
  if (ctx->nb > 1) return implicit_steps_batch(ctx, n, history);
  for (int64_t i = 0; i < n; ++i) {
    int rc = ctx->imp.prec ? implicit_step<float>(ctx, history ? history + i * 19 : nullptr)
                           : implicit_step<double>(ctx, history ? history + i * 19 : nullptr);
    if (rc) return rc;
  }
  IMP_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  prof_collect(ctx);
  return BES_OK;
}

int bes_profile(bes_ctx* ctx, int32_t enable, double* ms_out, int64_t* counts_out) {
  if (!ctx) return BES_ERR_INVALID;
  Profiler& P = ctx->prof;
  prof_collect(ctx);
  if (ms_out)
    for (int k = 0; k < PROF_NCAT; ++k) ms_out[k] = P.ms[k];
  if (counts_out)
    for (int k = 0; k < PROF_NCAT; ++k) counts_out[k] = P.count[k];
  for (int k = 0; k < PROF_NCAT; ++k) {
    P.ms[k] = 0;
    P.count[k] = 0;
  }
  P.on = enable != 0;
  return BES_OK;
}

int bes_implicit_assemble(bes_ctx* ctx, double cfl, double* rhs, double* blocks, int64_t* n_blocks) {
  if (!ctx) return BES_ERR_INVALID;
  if (ctx->opt.solver_type != 1 || !ctx->imp.A) return BES_ERR_INVALID;
  if (ctx->nb != 1) {
    ctx->last_error = "the system is assembled on single-condition contexts";
    return BES_ERR_UNSUPPORTED;
  }
  const SoaMesh& M = ctx->soa;
  const RefMesh& R = ctx->ref;
  const int64_t nc = M.nc;
  int64_t nb = 0;
  for (int64_t c = 0; c < nc; ++c) {
    nb += 1;
    for (int q = 0; q < 4; ++q) nb += R.cadj[c * 4 + q] >= 0;
  }
  if (n_blocks) *n_blocks = nb;
  if (!rhs && !blocks) return BES_OK;
  double norms[15];
  int rc = ctx->imp.prec ? assemble<float>(ctx, cfl, norms) : assemble<double>(ctx, cfl, norms);
  if (rc) return rc;
  IMP_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (rhs) {
    std::vector<double> h(5 * nc);
    IMP_TRY(ctx, cudaMemcpy(h.data(), ctx->imp.rhs, 5 * nc * sizeof(double), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < nc; ++i)
      for (int v = 0; v < 5; ++v) rhs[M.cell_new2ref[i] * 5 + v] = h[v * nc + i];
  }
  if (blocks) {
    std::vector<double> A(125 * nc);
    if (ctx->imp.prec) {
      std::vector<float> Af(125 * nc);
      IMP_TRY(ctx, cudaMemcpy(Af.data(), ctx->imp.A, Af.size() * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t k = 0; k < Af.size(); ++k) A[k] = Af[k];
    } else {
      IMP_TRY(ctx, cudaMemcpy(A.data(), ctx->imp.A, A.size() * sizeof(double), cudaMemcpyDeviceToHost));
    }
    // reference block order: row by reference cell, diagonal first, then neighbours in local
    // face order (CoefficientMatrix::initialize, src/CoefficientMatrix.cpp:141-160)
    int64_t k = 0;
    for (int64_t c = 0; c < nc; ++c) {
      const int64_t i = M.cell_ref2new[c];
      for (int s = 0; s < 5; ++s) {
        if (s > 0 && R.cadj[c * 4 + (s - 1)] < 0) continue;
        for (int q = 0; q < 25; ++q) blocks[k * 25 + q] = A[(size_t)(s * 25 + q) * nc + i];
        ++k;
      }
    }
  }
  return check_nan_public(ctx);
}

int bes_ilu_order(bes_ctx* ctx, int64_t* order) {
  if (!ctx || !order) return BES_ERR_INVALID;
  const SoaMesh& M = ctx->soa;
  for (int64_t i = 0; i < M.nc; ++i) order[M.ilu_pos[i]] = M.cell_new2ref[i];
  return BES_OK;
}

}  // extern "C"
