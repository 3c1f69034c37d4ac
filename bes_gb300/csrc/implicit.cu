// Implicit (backward-Euler) pseudo-time step on the GPU: SolverImplicit::timeStep_
// (src/SolverImplicit.cpp:293-345) with the AMGCL solve (src/CoefficientMatrix.cpp:210-325)
// replaced by right-preconditioned restarted GMRES with a block-Jacobi or block-ILU(0)
// preconditioner.  The system (Jacobian, preconditioner, Krylov vectors) is FP64 for the plain
// method or FP32 for the defect correction; the residual, right-hand side, update and norms
// are always FP64.
//
// Every condition of a context is a slot, and one implicit step of all slots is ONE CUDA graph
// launch: the residual of every slot (one launch per kernel, slots on the grid's y axis), then
// per slot the Jacobians, the assembly and the factorisation (inside an IF node that skips a
// frozen slot), then the linear solves of all slots together: a WHILE node over restart
// cycles whose body holds one IF node per Arnoldi step, the Arnoldi kernels batched over the
// slots and the GMRES bookkeeping (Hessenberg column, Givens rotations, least squares,
// restart and convergence) in small device kernels (krylov_kernels.cuh).  The host reads the
// step's norms and linear-solve statistics back once per step and runs the CFL control.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "context.hpp"
#include "krylov_kernels.cuh"

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

// Stride of the Krylov vectors of a slot: 5 nc values, at least four more (the two-chunk
// gathers of the last cell read up to three values past it), rounded up to 64 values.
inline int64_t basis_stride(int64_t nc) { return (5 * nc + 4 + 63) / 64 * 64; }

inline bool uses_ilu(const bes_ctx* c) { return c->opt.linear_solver == 1 || c->opt.linear_solver == 2; }

// Device views of the implicit buffers: T is the system's type, B the basis element type.
template <class T, class B>
struct Sys {
  bes_ctx* c;
  int nc, nslot;
  int64_t N, ldv, sV, sA, sDinv;
  T *A, *LU, *Dinv, *Dc, *b, *Z, *W, *X, *Vx;
  B* V;
  bool packed, basis16;
  __half2 *A16, *LU16, *D16;
  float *As, *LUs, *Ds;
  cudaStream_t s;  // the stream being captured (switched inside conditional bodies)
  dim3 vgrid;      // vector kernels: kRedBlocks blocks per slot
  int nthr;        // control kernels: one thread per slot, rounded up to a warp
  explicit Sys(bes_ctx* ctx) : c(ctx) {
    ImplicitBuffers& I = ctx->imp;
    nc = ctx->soa.nc;
    nslot = I.nslot;
    N = 5LL * nc;
    ldv = I.ldv;
    sV = I.sV;
    sA = I.sA;
    sDinv = I.sDinv;
    A = (T*)I.A;
    LU = (T*)I.LU;
    Dinv = (T*)I.Dinv;
    Dc = (T*)I.Dc;
    b = (T*)I.b;
    Z = (T*)I.Z;
    W = (T*)I.W;
    X = (T*)I.X;
    Vx = (T*)I.Vx;
    V = (B*)I.V;
    packed = I.packed;
    basis16 = I.basis16;
    A16 = (__half2*)I.A16;
    LU16 = (__half2*)I.LU16;
    D16 = (__half2*)I.D16;
    As = I.As;
    LUs = I.LUs;
    Ds = I.Ds;
    s = ctx->stream;
    vgrid = dim3(kRedBlocks, nslot);
    nthr = std::min(kMaxSlots, (nslot + 31) / 32 * 32);
  }
  // per-slot views
  SlotPtr<T> vec(T* p) const { return slots(p, ldv); }
  SlotPtr<const T> cvec(const T* p) const { return cslots(p, ldv); }
  SlotPtr<B> basis(int k) const { return slots(V + (int64_t)k * ldv, sV); }
  SlotPtr<const B> cbasis(int k) const { return cslots(V + (int64_t)k * ldv, sV); }
  SlotPtr<double> red() const { return slots(c->imp.red, 64 * c->imp.red_ld); }
  SlotPtr<const double> cred() const { return cslots(c->imp.red, 64 * c->imp.red_ld); }
  SlotPtr<double> dev(int off = 0) const { return slots(c->imp.gm.dev + off, (int64_t)kGsLd); }
  SlotPtr<const double> cdev() const { return cslots(c->imp.gm.dev, (int64_t)kGsLd); }
  SlotPtr<float> devf() const { return slots(c->imp.gm.devf, (int64_t)kGsLd); }
  SlotPtr<const float> cdevf() const { return cslots(c->imp.gm.devf, (int64_t)kGsLd); }
  // the preconditioner's input for Arnoldi step j: the basis vector, or its FP32 copy
  SlotPtr<const T> precond_in(int j) const {
    if constexpr (std::is_same<T, B>::value) return cslots((const T*)(V + (int64_t)j * ldv), sV);
    else return cvec(Vx);
  }
  // system arrays of slot k (the shared scratch when sA == 0)
  T* A_of(int k) const { return A + (int64_t)k * sA; }
  T* LU_of(int k) const { return LU + (int64_t)k * sA; }
  T* Dinv_of(int k) const { return Dinv + (int64_t)k * sDinv; }
};

// Kernel nodes of a graph (not descending into conditional bodies).
int64_t kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
  std::vector<cudaGraphNode_t> nodes(n);
  if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
  int64_t k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

// Timing stamps around a kernel category, in the profiled variant of the step graph only.
thread_local bool t_stamps = false;
void stamp(bes_ctx* c, cudaStream_t s, int cat, int begin) {
  if (!t_stamps) return;
  prof_stamp_kernel<<<1, 1, 0, s>>>(c->prof.dev, cat, begin);
}

// Add a conditional node (IF or WHILE on handle h) after the current capture dependencies of
// `parent` and start capturing its body on `child`.
int begin_conditional(bes_ctx* c, cudaStream_t parent, cudaStream_t child,
                      cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  IMP_TRY(c, cudaStreamGetCaptureInfo(parent, &st, nullptr, &g, &deps, nullptr, &nd));
  if (st != cudaStreamCaptureStatusActive) {
    c->last_error = "conditional node outside a capture";
    return BES_ERR_CUDA;
  }
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  IMP_TRY(c, cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
  IMP_TRY(c, cudaStreamUpdateCaptureDependencies(parent, &node, nullptr, 1,
                                                 cudaStreamSetCaptureDependencies));
  IMP_TRY(c, cudaStreamBeginCaptureToGraph(child, p.conditional.phGraph_out[0], nullptr, nullptr,
                                           0, cudaStreamCaptureModeRelaxed));
  return BES_OK;
}

// End the body's capture; *kernels receives its kernel node count.
int end_conditional(bes_ctx* c, cudaStream_t child, int64_t* kernels) {
  cudaGraph_t body = nullptr;
  IMP_TRY(c, cudaStreamEndCapture(child, &body));
  *kernels = kernel_nodes(body);
  return BES_OK;
}

// ---- Krylov side, batched over slots -----------------------------------------------------

// The colour stages of a sweep: colours 1..C-2 forward, the last colour's two solves fused,
// colours C-2..0 backward.  False if there are more stages than a persistent sweep holds.
bool sweep_plan(const SoaMesh& M, SweepPlan& P) {
  const int C = M.n_stages;
  if (C < 1 || 2 * C - 1 > kMaxStages) return false;
  P = SweepPlan();
  P.s1 = C > 1 ? M.stage_off[1] : M.stage_off[C];
  auto add = [&](int k, int kind) {
    P.r0[P.n] = M.stage_off[k];
    P.r1[P.n] = M.stage_off[k + 1];
    P.kind[P.n] = kind;
    ++P.n;
  };
  for (int k = 1; k < C - 1; ++k) add(k, 0);
  add(C - 1, 1);
  for (int k = C - 2; k >= 0; --k) add(k, 2);
  return true;
}

// One persistent launch of the whole colour sweep from `in` into Z (cooperative: every block
// of the grid is resident, which the grid barrier between colours needs).
template <class T, class B>
cudaError_t launch_persistent_sweep(const Sys<T, B>& S, cudaStream_t s, SlotPtr<const T> in,
                                    const int32_t* run) {
  bes_ctx* c = S.c;
  const ImplicitBuffers& I = c->imp;
  SweepPlan P;
  if (!sweep_plan(c->soa, P)) return cudaErrorInvalidConfiguration;
  SweepOps<T> O;
  std::memset(&O, 0, sizeof(O));
  if (S.packed) {
    O.H = cslots((const __half2*)S.LU16, 52LL * S.nc);
    O.HS = cslots((const float*)S.LUs, 4LL * S.nc);
    O.D = cslots((const __half2*)S.D16, 13LL * S.nc);
    O.DS = cslots((const float*)S.Ds, (int64_t)S.nc);
  } else {
    O.L = cslots((const T*)S.LU, S.sA);
    O.Dinv = cslots((const T*)S.Dinv, S.sDinv);
  }
  O.in = in;
  O.out = S.vec(S.Z);
  const GridSync gs{I.sync_count, I.sync_gen, I.sync_error};
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3(I.persistent_blocks);
  cfg.blockDim = dim3(128);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if constexpr (std::is_same<T, float>::value)
    if (S.packed)
      return cudaLaunchKernelEx(&cfg, ilu_sweep_persistent_kernel<float, true>, c->dm, P, O,
                                S.nslot, run, gs);
  return cudaLaunchKernelEx(&cfg, ilu_sweep_persistent_kernel<T, false>, c->dm, P, O, S.nslot,
                            run, gs);
}

// Z = M^{-1} in for every slot whose run flag is set
template <class T, class B>
void enqueue_precond(const Sys<T, B>& S, cudaStream_t s, SlotPtr<const T> in, const int32_t* run) {
  bes_ctx* c = S.c;
  const SoaMesh& M = c->soa;
  const DevMesh& m = c->dm;
  SlotPtr<T> Z = S.vec(S.Z);
  if (uses_ilu(c) && c->imp.use_colour_ranges && c->imp.sweep_kernel == 2) {
    launch_persistent_sweep(S, s, in, run);
    return;
  }
  if (!uses_ilu(c)) {
    if constexpr (std::is_same<T, float>::value) {
      if (S.packed) {
        jacobi_apply_packed_kernel<<<dim3(nblk(S.nc, 256), S.nslot), 256, 0, s>>>(
            S.nc, cslots((const __half2*)S.D16, 13LL * S.nc), cslots((const float*)S.Ds, (int64_t)S.nc),
            in, Z, run);
        return;
      }
    }
    jacobi_apply_kernel<T><<<dim3(nblk(S.nc, 256), S.nslot), 256, 0, s>>>(
        S.nc, cslots((const T*)S.Dinv, S.sDinv), in, Z, run);
    return;
  }
  if (c->imp.use_colour_ranges) {
    // colours 1..C-2 forward, the last colour's two solves fused, colours C-2..0 backward
    const int C = M.n_stages;
    const int s1 = M.stage_off[1];
    auto launch = [&](int k, bool lower, bool upper) {
      const int r0 = M.stage_off[k], r1 = M.stage_off[k + 1];
      const dim3 grid(nblk(r1 - r0, 128), S.nslot);
      if constexpr (std::is_same<T, float>::value) {
        if (S.packed) {
          auto H = cslots((const __half2*)S.LU16, 52LL * S.nc);
          auto HS = cslots((const float*)S.LUs, 4LL * S.nc);
          auto D = cslots((const __half2*)S.D16, 13LL * S.nc);
          auto DS = cslots((const float*)S.Ds, (int64_t)S.nc);
#define BES_PACKED_SWEEP(LO, UP, BA)                                                          \
  do {                                                                                        \
    if (c->imp.sweep_kernel == 3)                                                             \
      ilu_colour_packed_ld_kernel<LO, UP, BA><<<grid, 128, 0, s>>>(m, r0, r1, s1, H, HS, D, DS, \
                                                                   in, Z, run);               \
    else                                                                                      \
      ilu_colour_packed_kernel<LO, UP, BA><<<grid, 128, 0, s>>>(m, r0, r1, s1, H, HS, D, DS,   \
                                                                in, Z, run);                  \
  } while (0)
          if (S.nslot > 1) {
            if (lower && !upper) BES_PACKED_SWEEP(true, false, true);
            else if (lower) BES_PACKED_SWEEP(true, true, true);
            else BES_PACKED_SWEEP(false, true, true);
          } else {
            if (lower && !upper) BES_PACKED_SWEEP(true, false, false);
            else if (lower) BES_PACKED_SWEEP(true, true, false);
            else BES_PACKED_SWEEP(false, true, false);
          }
#undef BES_PACKED_SWEEP
          return;
        }
      }
      auto L = cslots((const T*)S.LU, S.sA);
      auto D = cslots((const T*)S.Dinv, S.sDinv);
#define BES_SWEEP(LO, UP, BA) \
  ilu_colour_kernel<T, LO, UP, BA><<<grid, 128, 0, s>>>(m, r0, r1, s1, L, D, in, Z, run)
      if (S.nslot > 1) {
        if (lower && !upper) BES_SWEEP(true, false, true);
        else if (lower) BES_SWEEP(true, true, true);
        else BES_SWEEP(false, true, true);
      } else {
        if (lower && !upper) BES_SWEEP(true, false, false);
        else if (lower) BES_SWEEP(true, true, false);
        else BES_SWEEP(false, true, false);
      }
#undef BES_SWEEP
    };
    for (int k = 1; k < C - 1; ++k) launch(k, true, false);
    launch(C - 1, true, true);
    for (int k = C - 2; k >= 0; --k) launch(k, false, true);
    return;
  }
  // level-scheduled stages (RCM order), in place on Z
  copy_vec_kernel<T><<<S.vgrid, 256, 0, s>>>(Z, in, S.N, run);
  auto L = cslots((const T*)S.LU, S.sA);
  auto D = cslots((const T*)S.Dinv, S.sDinv);
  for (int k = 0; k < M.n_stages; ++k) {
    const int n = M.stage_off[k + 1] - M.stage_off[k];
    ilu_lower_kernel<T><<<dim3(nblk(n, 128), S.nslot), 128, 0, s>>>(
        m, c->imp.stage_rows + M.stage_off[k], n, c->imp.ilu_pos, L, Z, run);
  }
  for (int k = M.n_stages - 1; k >= 0; --k) {
    const int n = M.stage_off[k + 1] - M.stage_off[k];
    ilu_upper_kernel<T><<<dim3(nblk(n, 128), S.nslot), 128, 0, s>>>(
        m, c->imp.stage_rows + M.stage_off[k], n, c->imp.ilu_pos, L, D, Z, run);
  }
}

// y = A x, or y = b - A x when b is given
template <class T, class B>
void enqueue_spmv(const Sys<T, B>& S, cudaStream_t s, SlotPtr<const T> x, SlotPtr<const T> b,
                  SlotPtr<T> y, const int32_t* run) {
  const dim3 grid(nblk(S.nc, 256), S.nslot);
  if constexpr (std::is_same<T, float>::value) {
    if (S.packed) {
      auto H = cslots((const __half2*)S.A16, 65LL * S.nc);
      auto Sc = cslots((const float*)S.As, 5LL * S.nc);
      if (S.nslot > 1)
        spmv_packed_kernel<true><<<grid, 256, 0, s>>>(S.c->dm, H, Sc, x, b, y, run);
      else
        spmv_packed_kernel<false><<<grid, 256, 0, s>>>(S.c->dm, H, Sc, x, b, y, run);
      return;
    }
  }
  if (S.nslot > 1)
    spmv_kernel<T, true><<<grid, 256, 0, s>>>(S.c->dm, cslots((const T*)S.A, S.sA), x, b, y, run);
  else
    spmv_kernel<T, false><<<grid, 256, 0, s>>>(S.c->dm, cslots((const T*)S.A, S.sA), x, b, y, run);
}

// Body of the IF node of Arnoldi step j (slots with a running cycle): w = A M^{-1} v_j,
// Gram-Schmidt against v_0..v_j, v_{j+1}, and the Givens update of the Hessenberg column.
template <class T, class B>
int enqueue_arnoldi(const Sys<T, B>& S, cudaStream_t s, int j, const GmresParam& P,
                    const GmresHandles& h, int64_t* gs2_kernels) {
  bes_ctx* c = S.c;
  // with one slot the IF node alone decides whether the step runs: no per-block flag load
  const int32_t* cyc = S.nslot > 1 ? c->imp.gm.cyc : nullptr;
  const int nv = j + 1;
  stamp(c, s, PROF_PRECOND, 1);
  enqueue_precond(S, s, S.precond_in(j), cyc);
  stamp(c, s, PROF_PRECOND, 0);
  stamp(c, s, PROF_SPMV, 1);
  enqueue_spmv(S, s, S.cvec(S.Z), SlotPtr<const T>{nullptr, 0}, S.vec(S.W), cyc);
  stamp(c, s, PROF_SPMV, 0);
  stamp(c, s, PROF_ORTHO, 1);
  const auto Vb = S.cbasis(0);
  launch_gs_dots<T, B>(nv, S.vgrid, s, Vb, S.ldv, S.cvec(S.W), S.N, S.red(), cyc);
  reduce_slots_kernel<<<dim3(nv + 1, S.nslot), 256, 0, s>>>(S.cred(), kRedBlocks, nv + 1, 0,
                                                            S.dev(), cyc);
  gs_decide_kernel<<<dim3(1, S.nslot), 64, 0, s>>>(S.dev(), S.devf(), nv, 1, cyc, h.gs2[j],
                                                    h.on, nullptr);
  launch_gs_update<T, B, GS_FINAL1>(nv, S.vgrid, s, S.basis(j + 1), S.vec(S.Vx), S.vec(S.W), Vb,
                                    S.ldv, S.cdev(), S.cdevf(), S.N, S.red(), cyc);
  // the second pass (rare): in the step graph an IF node that runs only when a slot needs it,
  // so that its four launches cost nothing otherwise
  cudaStream_t s2 = s;
  if (h.on) {
    s2 = c->imp.cap[2];
    if (const int rc = begin_conditional(c, s, s2, h.gs2[j], cudaGraphCondTypeIf)) return rc;
  }
  launch_gs_update<T, B, GS_REORTH>(nv, S.vgrid, s2, S.basis(j + 1), S.vec(S.Vx), S.vec(S.W), Vb,
                                    S.ldv, S.cdev(), S.cdevf(), S.N, S.red(), cyc);
  reduce_slots_kernel<<<dim3(nv + 1, S.nslot), 256, 0, s2>>>(S.cred(), kRedBlocks, nv + 1, 0,
                                                             S.dev(kGsH2), cyc);
  gs_decide_kernel<<<dim3(1, S.nslot), 64, 0, s2>>>(S.dev(), S.devf(), nv, 2, cyc, h.gs2[j],
                                                     h.on, h.on ? c->imp.gm.counters + 2 : nullptr);
  launch_gs_update<T, B, GS_FINAL2>(nv, S.vgrid, s2, S.basis(j + 1), S.vec(S.Vx), S.vec(S.W), Vb,
                                    S.ldv, S.cdev(), S.cdevf(), S.N, S.red(), cyc);
  if (h.on) {
    if (const int rc = end_conditional(c, s2, gs2_kernels)) return rc;
  }
  gmres_givens_kernel<<<1, S.nthr, 0, s>>>(c->imp.gm, P, h, S.nslot, j);
  stamp(c, s, PROF_ORTHO, 0);
  return BES_OK;
}

// End of a restart cycle (slots whose solve runs): x += M^{-1} V y, r = b - A x, and the
// restart decision; the next cycle's v_0 = r / |r|.
template <class T, class B>
void enqueue_cycle_end(const Sys<T, B>& S, cudaStream_t s, const GmresParam& P,
                       const GmresHandles& h) {
  bes_ctx* c = S.c;
  const GmresDev& g = c->imp.gm;
  // with one slot the WHILE node alone decides whether the cycle end runs
  const int32_t* lin = S.nslot > 1 ? g.lin : nullptr;
  stamp(c, s, PROF_ORTHO, 1);
  gmres_solve_y_kernel<<<1, S.nthr, 0, s>>>(g, S.nslot);
  lincomb_kernel<T, B><<<S.vgrid, 256, 0, s>>>(S.vec(S.W), S.cbasis(0), S.ldv, g.jc,
                                               cslots((const double*)g.y, (int64_t)kMaxRestart),
                                               S.N, lin);
  stamp(c, s, PROF_ORTHO, 0);
  stamp(c, s, PROF_PRECOND, 1);
  enqueue_precond(S, s, S.cvec(S.W), lin);
  stamp(c, s, PROF_PRECOND, 0);
  stamp(c, s, PROF_SPMV, 1);
  add_kernel<T><<<S.vgrid, 256, 0, s>>>(S.vec(S.X), S.cvec(S.Z), S.N, lin);
  enqueue_spmv(S, s, S.cvec(S.X), S.cvec(S.b), S.vec(S.W), lin);
  stamp(c, s, PROF_SPMV, 0);
  stamp(c, s, PROF_ORTHO, 1);
  norm2_kernel<T><<<S.vgrid, 256, 0, s>>>(S.cvec(S.W), S.N, S.red(), lin);
  reduce_slots_kernel<<<dim3(1, S.nslot), 256, 0, s>>>(S.cred(), kRedBlocks, 1, 0, S.dev(kGsR),
                                                       lin);
  gmres_restart_kernel<<<1, S.nthr, 0, s>>>(g, P, h, S.nslot, c->imp.guard_dev);
  basis_start_kernel<T, B><<<S.vgrid, 256, 0, s>>>(S.basis(0), S.vec(S.Vx), S.cvec(S.W),
                                                   cslots((const double*)g.sc, 8LL), S.N, g.cyc);
  stamp(c, s, PROF_ORTHO, 0);
}

// Start of the linear solves of the slots taking the step: x = 0, beta = |b|, v_0 = b / beta.
template <class T, class B>
void enqueue_solve_init(const Sys<T, B>& S, cudaStream_t s, const GmresParam& P,
                        const GmresHandles& h) {
  bes_ctx* c = S.c;
  const GmresDev& g = c->imp.gm;
  const int32_t* act = c->imp.act;
  stamp(c, s, PROF_ORTHO, 1);
  zero_kernel<T><<<S.vgrid, 256, 0, s>>>(S.vec(S.X), S.N, act);
  norm2_kernel<T><<<S.vgrid, 256, 0, s>>>(S.cvec(S.b), S.N, S.red(), act);
  reduce_slots_kernel<<<dim3(1, S.nslot), 256, 0, s>>>(S.cred(), kRedBlocks, 1, 0, S.dev(kGsR), act);
  gmres_init_kernel<<<1, S.nthr, 0, s>>>(g, P, h, S.nslot, act, c->nan_flag);
  basis_start_kernel<T, B><<<S.vgrid, 256, 0, s>>>(S.basis(0), S.vec(S.Vx), S.cvec(S.b),
                                                   cslots((const double*)g.sc, 8LL), S.N, g.lin);
  stamp(c, s, PROF_ORTHO, 0);
}

// ---- assembly and factorisation, slot by slot ----------------------------------------------

// Residual of every slot taking the step (explicit stage-0 kernels, slots on the grid's y
// axis): local or global time step at the slot's CFL, face-side states, face fluxes.
void enqueue_residual_all(bes_ctx* c, cudaStream_t s, const SlotHandles& hs, int on) {
  const DevMesh& m = c->dm;
  const int nslot = c->imp.nslot;
  step_begin_kernel<<<1, 256, 0, s>>>(hs, on, nslot, c->imp.act, c->dtmin);
  Params prm = c->prm;
  prm.active = c->imp.act;
  stamp(c, s, PROF_RESIDUAL, 1);
  cell_recon_kernel<true, false><<<dim3(nblk(m.nc, kBlock), nslot), kBlock, 0, s>>>(
      m, prm, c->U[c->cur], c->RS, c->rs_ld, c->dt, 0.0, c->opt.local_time_step, c->dtmin,
      nullptr, nullptr, c->imp.cfl_dev);
  face_flux_kernel<false><<<dim3(nblk(m.nf, kBlock), nslot), kBlock, 0, s>>>(
      m, prm, c->RS, c->rs_ld, c->FA, nullptr, c->nan_flag);
  stamp(c, s, PROF_RESIDUAL, 0);
}

// 16-bit block-scaled copies (precision 2; T is float there)
template <class T>
void enqueue_pack(cudaStream_t s, int nc, const T* src, int slot0, int nslots, void* H, float* sc) {
  if constexpr (std::is_same<T, float>::value)
    pack_blocks_kernel<<<dim3(nblk(nc, 256), nslots), 256, 0, s>>>(src, slot0, nc, (__half2*)H, sc);
}

// Slot k: first-order Jacobians, the assembled system with its right-hand side, the 16-bit
// copies (precision 2) and the step's norms (into norms [15]: L2 of the right-hand side [5],
// L2 of R [5], max of the right-hand side [5]).
template <class T, class B>
void enqueue_assembly(const Sys<T, B>& S, cudaStream_t s, int k, double* norms) {
  bes_ctx* c = S.c;
  const DevMesh& m = c->dm;
  const bes_options& o = c->opt;
  const int64_t nc = m.nc, nf = m.nf;
  const int local = o.local_time_step;
  const double* U = c->U[c->cur] + k * 5 * nc;
  const double* dt = c->dt + k * nc;
  const unsigned long long* dtmin = c->dtmin + k;
  Params prm = c->prm;
  prm.pinf_dev = c->pinf_dev + 6 * k;
  prm.active = nullptr;
  FaceLocal fl{c->imp.m_own, c->imp.m_nb};
  T* A = S.A_of(k);
  T* Dinv = S.Dinv_of(k);
  double* red = c->imp.red + (int64_t)k * 64 * c->imp.red_ld;
  stamp(c, s, PROF_JACOBIAN, 1);
  face_jacobian_kernel<T><<<nblk(nf, 128), 128, 0, s>>>(m, prm, fl, U, dt, dtmin, local,
                                                        o.jacobian_repeat, A, S.Dc);
  stamp(c, s, PROF_JACOBIAN, 0);
  stamp(c, s, PROF_ASSEMBLE, 1);
  const int nb = nblk(nc, 128);
  cell_assemble_kernel<T><<<nb, 128, 0, s>>>(m, c->FA + k * 5 * nf, dt, dtmin, local,
                                             o.jacobian_repeat, S.Dc, A,
                                             uses_ilu(c) ? nullptr : Dinv,
                                             c->imp.rhs + k * 5 * nc, S.b + k * S.ldv, red);
  if (S.packed) {
    enqueue_pack(s, (int)nc, A, 0, 5, S.A16 + k * 65 * nc, S.As + k * 5 * nc);
    if (!uses_ilu(c)) enqueue_pack(s, (int)nc, Dinv, 0, 1, S.D16 + k * 13 * nc, S.Ds + k * nc);
  }
  reduce_rows_kernel<<<15, 256, 0, s>>>(red, nb, 10, 1, norms);
  stamp(c, s, PROF_ASSEMBLE, 0);
}

// Slot k: block-ILU(0) factorisation of a copy of A, stage by stage (the factorisation of the
// stage's rows, then the inverses of their diagonal blocks), and its 16-bit copies.
template <class T, class B>
void enqueue_factor(const Sys<T, B>& S, cudaStream_t s, int k) {
  bes_ctx* c = S.c;
  if (!uses_ilu(c)) return;
  const SoaMesh& M = c->soa;
  const int64_t nc = S.nc;
  T* LU = S.LU_of(k);
  T* Dinv = S.Dinv_of(k);
  stamp(c, s, PROF_ILU_FACTOR, 1);
  copy_vec_kernel<T><<<dim3(kRedBlocks, 1), 256, 0, s>>>(slots(LU, 0), cslots((const T*)S.A_of(k), 0),
                                                        125 * nc, nullptr);
  for (int q = 0; q < M.n_stages; ++q) {
    const int n = M.stage_off[q + 1] - M.stage_off[q];
    if (c->imp.use_colour_ranges) {
      ilu_factor_kernel<T, true><<<nblk(n, 128), 128, 0, s>>>(c->dm, nullptr, n, nullptr, LU, Dinv,
                                                              M.stage_off[q]);
      ilu_invert_kernel<T, true><<<nblk(n, 128), 128, 0, s>>>(c->dm, nullptr, n, LU, Dinv,
                                                              M.stage_off[q]);
    } else {
      ilu_factor_kernel<T><<<nblk(n, 128), 128, 0, s>>>(c->dm, c->imp.stage_rows + M.stage_off[q],
                                                        n, c->imp.ilu_pos, LU, Dinv);
      ilu_invert_kernel<T><<<nblk(n, 128), 128, 0, s>>>(c->dm, c->imp.stage_rows + M.stage_off[q],
                                                        n, LU, Dinv);
    }
  }
  if (S.packed) {
    enqueue_pack(s, (int)nc, LU, 1, 4, S.LU16 + k * 52 * nc, S.LUs + k * 4 * nc);
    enqueue_pack(s, (int)nc, Dinv, 0, 1, S.D16 + k * 13 * nc, S.Ds + k * nc);
  }
  stamp(c, s, PROF_ILU_FACTOR, 0);
}

// ---- autotuner ------------------------------------------------------------------------------

int reset_grid_sync(bes_ctx* c) {
  ImplicitBuffers& I = c->imp;
  IMP_TRY(c, cudaMemsetAsync(I.sync_count, 0, sizeof(unsigned), c->stream));
  IMP_TRY(c, cudaMemsetAsync(I.sync_gen, 0, sizeof(unsigned), c->stream));
  IMP_TRY(c, cudaMemsetAsync(I.sync_error, 0, sizeof(int), c->stream));
  IMP_TRY(c, cudaStreamSynchronize(c->stream));
  return BES_OK;
}

// The colour-sweep variant, timed on this context's mesh and slots: one launch per colour, or
// one persistent launch per sweep.  Each candidate runs 3 untimed and 10 timed sweeps (CUDA
// events on the context's stream, all slots); a persistent candidate whose launch fails or
// whose grid barrier gives up is dropped.  The options can fix the variant instead.
template <class T, class B>
int tune_sweep(bes_ctx* c) {
  ImplicitBuffers& I = c->imp;
  Sys<T, B> S(c);
  I.tuned = true;
  char line[256];
  if (!uses_ilu(c) || !I.use_colour_ranges) {
    I.sweep_kernel = 1;
    return BES_OK;
  }
  SweepPlan plan;
  const bool can_persist = sweep_plan(c->soa, plan) && I.persistent_blocks > 0;
  static const char* kNames[4] = {"", "one launch per colour", "persistent",
                                  "one launch per colour, loads first"};
  if (c->opt.sweep_kernel >= 1 && c->opt.sweep_kernel <= 3) {
    I.sweep_kernel = c->opt.sweep_kernel;
    if (I.sweep_kernel == 2 && !can_persist) I.sweep_kernel = 1;
    if (I.sweep_kernel == 3 && !I.packed) I.sweep_kernel = 1;
    std::snprintf(line, sizeof(line), "colour sweep: %s (fixed by the options)\n",
                  kNames[I.sweep_kernel]);
    I.tuning += line;
    return BES_OK;
  }
  cudaEvent_t e0, e1;
  IMP_TRY(c, cudaEventCreate(&e0));
  IMP_TRY(c, cudaEventCreate(&e1));
  double best = 1e300;
  int choice = 1;
  std::string rep = "colour sweep:";
  for (int cand = 1; cand <= 3; ++cand) {
    if (cand == 2 && !can_persist) {
      rep += " persistent not possible;";
      continue;
    }
    if (cand == 3 && !I.packed) continue;  // a form of the 16-bit storage only
    I.sweep_kernel = cand;
    bool ok = true;
    float ms = 0.0f;
    for (int r = 0; r < 13 && ok; ++r) {
      if (r == 3) cudaEventRecord(e0, c->stream);
      if (cand == 2)
        ok = launch_persistent_sweep(S, c->stream, S.cvec(S.b), nullptr) == cudaSuccess;
      else
        enqueue_precond(S, c->stream, S.cvec(S.b), nullptr);
    }
    cudaEventRecord(e1, c->stream);
    const cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      c->last_error = std::string("colour-sweep tuning: ") + cudaGetErrorString(e);
      return BES_ERR_CUDA;
    }
    if (ok) {
      cudaEventElapsedTime(&ms, e0, e1);
      if (cand == 2) {
        int err = 0;
        cudaMemcpy(&err, I.sync_error, sizeof(int), cudaMemcpyDeviceToHost);
        if (err) ok = false;
      }
    }
    // a refused launch leaves no sticky error; its form is dropped
    if (cudaGetLastError() != cudaSuccess) ok = false;
    if (cand == 2) {
      const int rc = reset_grid_sync(c);
      if (rc) return rc;
    }
    const double per = ms / 10.0;
    if (cand != 2 && ok)
      std::snprintf(line, sizeof(line), " %s %.4f ms;", kNames[cand], per);
    else if (cand != 2)
      std::snprintf(line, sizeof(line), " %s failed;", kNames[cand]);
    else if (ok)
      std::snprintf(line, sizeof(line), " persistent (%d blocks of 128) %.4f ms;",
                    I.persistent_blocks, per);
    else
      std::snprintf(line, sizeof(line), " persistent failed;");
    rep += line;
    if (ok && per < best) {
      best = per;
      choice = cand;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  I.sweep_kernel = choice;
  std::snprintf(line, sizeof(line), " taken: %s (%d slots, %d cells)\n", kNames[choice],
                S.nslot, S.nc);
  rep += line;
  I.tuning += rep;
  return BES_OK;
}

// ---- the step graph -------------------------------------------------------------------------

// Device address of slot k's norms in the device array of step results.
double* result_norms(StepResult* res, int k) {
  return reinterpret_cast<double*>(reinterpret_cast<char*>(res + k) + offsetof(StepResult, norms));
}

// End every capture still open after a failure, so the streams are usable again.
void abandon_capture(bes_ctx* c) {
  cudaStream_t ss[4] = {c->imp.cap[2], c->imp.cap[1], c->imp.cap[0], c->stream};
  for (cudaStream_t s : ss) {
    cudaStreamCaptureStatus st;
    if (s && cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
    }
  }
  cudaGetLastError();
}

template <class T, class B>
int capture_step(bes_ctx* c, int prof, cudaGraph_t* out) {
  Sys<T, B> S(c);
  ImplicitBuffers& I = c->imp;
  const bes_options& o = c->opt;
  cudaStream_t s0 = c->stream, s1 = I.cap[0], s2 = I.cap[1];
  IMP_TRY(c, cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed));
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  IMP_TRY(c, cudaStreamGetCaptureInfo(s0, &st, nullptr, &g, nullptr, nullptr, nullptr));
  SlotHandles hs;
  std::memset(&hs, 0, sizeof(hs));
  for (int k = 0; k < S.nslot; ++k)
    IMP_TRY(c, cudaGraphConditionalHandleCreate(&hs.h[k], g, 0, cudaGraphCondAssignDefault));
  GmresHandles gh;
  std::memset(&gh, 0, sizeof(gh));
  gh.on = 1;
  IMP_TRY(c, cudaGraphConditionalHandleCreate(&gh.loop, g, 0, cudaGraphCondAssignDefault));
  for (int j = 0; j < o.gmres_restart; ++j) {
    IMP_TRY(c, cudaGraphConditionalHandleCreate(&gh.arn[j], g, 0, cudaGraphCondAssignDefault));
    IMP_TRY(c, cudaGraphConditionalHandleCreate(&gh.gs2[j], g, 0, cudaGraphCondAssignDefault));
  }
  const GmresParam P{o.gmres_restart, o.linear_solver_max_iter, o.linear_solver_tol};
  int rc;
  enqueue_residual_all(c, s0, hs, 1);
  for (int k = 0; k < S.nslot; ++k) {
    if ((rc = begin_conditional(c, s0, s1, hs.h[k], cudaGraphCondTypeIf))) return rc;
    enqueue_assembly(S, s1, k, result_norms(I.res, k));
    enqueue_factor(S, s1, k);
    if ((rc = end_conditional(c, s1, &I.nodes_slot[prof]))) return rc;
  }
  enqueue_solve_init(S, s0, P, gh);
  if ((rc = begin_conditional(c, s0, s1, gh.loop, cudaGraphCondTypeWhile))) return rc;
  for (int j = 0; j < o.gmres_restart; ++j) {
    if ((rc = begin_conditional(c, s1, s2, gh.arn[j], cudaGraphCondTypeIf))) return rc;
    if ((rc = enqueue_arnoldi(S, s2, j, P, gh, &I.nodes_gs2[prof]))) return rc;
    if ((rc = end_conditional(c, s2, &I.nodes_arn[prof]))) return rc;
  }
  enqueue_cycle_end(S, s1, P, gh);
  if ((rc = end_conditional(c, s1, &I.nodes_loop[prof]))) return rc;
  gmres_finish_kernel<<<1, S.nthr, 0, s0>>>(I.gm, I.res, S.nslot, I.act);
  stamp(c, s0, PROF_OTHER, 1);
  state_update_kernel<T><<<S.vgrid, 256, 0, s0>>>(slots(c->U[c->cur], 5LL * S.nc), S.cvec(S.X),
                                                  (int64_t)S.nc, c->nan_flag, I.act);
  stamp(c, s0, PROF_OTHER, 0);
  IMP_TRY(c, cudaGetLastError());
  IMP_TRY(c, cudaStreamEndCapture(s0, out));
  I.nodes_top[prof] = kernel_nodes(*out);
  return BES_OK;
}

template <class T, class B>
int build_step_graph(bes_ctx* c, int prof) {
  ImplicitBuffers& I = c->imp;
  if (!I.cap[0]) {
    IMP_TRY(c, cudaStreamCreateWithFlags(&I.cap[0], cudaStreamNonBlocking));
    IMP_TRY(c, cudaStreamCreateWithFlags(&I.cap[1], cudaStreamNonBlocking));
    IMP_TRY(c, cudaStreamCreateWithFlags(&I.cap[2], cudaStreamNonBlocking));
  }
  if (!I.tuned) {
    const int rc = tune_sweep<T, B>(c);
    if (rc) return rc;
  }
  cudaGraph_t g = nullptr;
  t_stamps = prof != 0;
  int rc = capture_step<T, B>(c, prof, &g);
  if (rc && I.sweep_kernel == 2) {
    // the persistent launch could not be captured: one launch per colour
    abandon_capture(c);
    I.sweep_kernel = 1;
    I.tuning += "colour sweep: the persistent launch could not be captured in the step graph; "
                "taken: one launch per colour\n";
    rc = capture_step<T, B>(c, prof, &g);
  }
  t_stamps = false;
  if (rc) {
    abandon_capture(c);
    return rc;
  }
  const cudaError_t e = cudaGraphInstantiate(&I.step_graph[prof][c->cur], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    c->last_error = std::string("cudaGraphInstantiate (implicit step): ") + cudaGetErrorString(e);
    I.step_graph[prof][c->cur] = nullptr;
    return BES_ERR_CUDA;
  }
  return BES_OK;
}

// ---- host side of a step -------------------------------------------------------------------

double cfl_for_step(const bes_options& o, const SlotCtl& k) {
  if (o.cfl_ramp_steps > 0) {
    if (k.step_count >= o.cfl_ramp_steps - 1 || o.cfl_ramp_steps == 1) return o.cfl_ramp_end;
    const double t = (double)k.step_count / (double)(o.cfl_ramp_steps - 1);
    return o.cfl_ramp_start * std::pow(o.cfl_ramp_end / o.cfl_ramp_start, t);
  }
  return k.cfl_actual;
}

int check_step_nan(bes_ctx* c, int flag) {
  if (!flag) return BES_OK;
  IMP_TRY(c, cudaMemsetAsync(c->nan_flag, 0, sizeof(int), c->stream));
  IMP_TRY(c, cudaStreamSynchronize(c->stream));
  const int64_t f = c->soa.face_new2ref[flag - 1];
  char buf[256];
  std::snprintf(buf, sizeof(buf),
                "NaN values encountered in flux across face %lld at coordinates [%e, %e, %e]",
                (long long)f, c->ref.center[f * 3], c->ref.center[f * 3 + 1],
                c->ref.center[f * 3 + 2]);
  c->last_error = buf;
  return BES_ERR_NAN;
}

// Upload the step's per-slot inputs: which slots step, their CFL and ramped freestream.
int upload_step_inputs(bes_ctx* c, std::vector<int32_t>& act, std::vector<double>& cfl,
                       std::vector<double>& P) {
  ImplicitBuffers& I = c->imp;
  const int ns = I.nslot;
  act.assign(ns, 0);
  cfl.assign(ns, 0.0);
  P.assign(6 * ns, 0.0);
  for (int k = 0; k < ns; ++k) {
    act[k] = c->active_host[k] ? 1 : 0;
    const SlotCtl& t = I.ctl[k];
    cfl[k] = cfl_for_step(c->opt, t);
    // FREESTREAM_RAMP (Config::getFreestreamPrimitiveVariables, src/Config.cpp:688-706)
    freestream_from(&c->pinf0_host[6 * k], c->prm.ramp_steps, c->prm.ramp_frac, t.host_step,
                    &P[6 * k]);
  }
  IMP_TRY(c, cudaMemcpyAsync(I.act, act.data(), ns * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  IMP_TRY(c, cudaMemcpyAsync(I.cfl_dev, cfl.data(), ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  IMP_TRY(c, cudaMemcpyAsync(c->pinf_dev, P.data(), P.size() * sizeof(double),
                             cudaMemcpyHostToDevice, c->stream));
  return BES_OK;
}

// n implicit steps of every active slot; history [n][nslot][19]
template <class T, class B>
int run_steps(bes_ctx* c, int64_t n, double* history) {
  ImplicitBuffers& I = c->imp;
  const bes_options& o = c->opt;
  const int prof = c->prof.on ? 1 : 0;
  const int ns = I.nslot;
  if (!I.step_graph[prof][c->cur]) {
    const int rc = build_step_graph<T, B>(c, prof);
    if (rc) return rc;
  }
  std::vector<int32_t> act;
  std::vector<double> cfl, P;
  for (int64_t i = 0; i < n; ++i) {
    int rc = upload_step_inputs(c, act, cfl, P);
    if (rc) return rc;
    IMP_TRY(c, cudaGraphLaunch(I.step_graph[prof][c->cur], c->stream));
    int nan = 0, sync_err = 0;
    unsigned long long cnt[3];
    IMP_TRY(c, cudaMemcpyAsync(I.res_host.data(), I.res, ns * sizeof(StepResult),
                               cudaMemcpyDeviceToHost, c->stream));
    IMP_TRY(c, cudaMemcpyAsync(cnt, I.gm.counters, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
    IMP_TRY(c, cudaMemcpyAsync(&nan, c->nan_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    IMP_TRY(c, cudaMemcpyAsync(&sync_err, I.sync_error, sizeof(int), cudaMemcpyDeviceToHost,
                               c->stream));
    IMP_TRY(c, cudaStreamSynchronize(c->stream));
    ++I.host_syncs;
    if (sync_err) {
      if ((rc = reset_grid_sync(c))) return rc;
      c->last_error = "a grid barrier of the persistent colour sweep gave up after one second; "
                      "the step's linear solves are not valid";
      return BES_ERR_TIMEOUT;
    }
    // kernels this step launched: the graph's top level, the assembly of each slot that
    // stepped, and the Arnoldi and restart-cycle bodies the device ran
    int nact = 0;
    for (int k = 0; k < ns; ++k) nact += act[k];
    c->launches += I.nodes_top[prof] + nact * I.nodes_slot[prof] +
                   (int64_t)(cnt[0] - I.counters_host[0]) * I.nodes_arn[prof] +
                   (int64_t)(cnt[1] - I.counters_host[1]) * I.nodes_loop[prof] +
                   (int64_t)(cnt[2] - I.counters_host[2]) * I.nodes_gs2[prof];
    for (int q = 0; q < 3; ++q) I.counters_host[q] = cnt[q];
    if ((rc = check_step_nan(c, nan))) return rc;
    int status = BES_OK;
    for (int k = 0; k < ns; ++k) {
      double* h = history ? history + (i * ns + k) * 19 : nullptr;
      if (h) std::fill(h, h + 19, 0.0);
      if (!act[k]) continue;
      const StepResult& r = I.res_host[k];
      SlotCtl& t = I.ctl[k];
      // reduced rows: L2 of the right-hand side [5], L2 of R [5], max of the right-hand side [5]
      double norms[15];
      for (int v = 0; v < 5; ++v) {
        norms[v] = r.norms[v];
        norms[5 + v] = r.norms[10 + v];
        norms[10 + v] = r.norms[5 + v];
      }
      for (int v = 0; v < 5; ++v) {
        t.maxres_old[v] = t.maxres[v];
        t.maxres[v] = norms[5 + v];
      }
      if (o.cfl_ramp_steps <= 0 && o.adaptive_courant_num_max > o.courant_num) {
        // SolverImplicit::adaptCourantNum_ (src/SolverImplicit.cpp:530-550)
        const int idx = (t.maxres_old[0] > t.maxres[0]) ? 1 : 0;
        t.cfl_actual *= std::pow(t.maxres_old[0] / t.maxres[0], o.adaptive_courant_num_exponent[idx]);
        t.cfl_actual = std::max(o.courant_num, t.cfl_actual);
        t.cfl_actual = std::min(o.adaptive_courant_num_max, t.cfl_actual);
      }
      I.last_iters = r.iters;
      I.last_err = r.rel;
      I.total_lin_iters += r.iters;
      I.gs_second_passes += r.second;
      if (r.status != BES_OK) status = r.status;
      if (h) {
        for (int q = 0; q < 10; ++q) h[q] = norms[q];
        h[10] = cfl[k];
        h[11] = t.cfl_actual;
        h[12] = r.iters;
        h[13] = r.rel;
        for (int q = 0; q < 5; ++q) h[14 + q] = norms[10 + q];
      }
      ++t.step_count;
      ++t.host_step;
    }
    ++I.step_count;
    if (status != BES_OK) {
      c->last_error = "a linear solve was stopped after its restart-cycle limit";
      return status;
    }
  }
  return BES_OK;
}

template <class T>
int run_steps_t(bes_ctx* c, int64_t n, double* history) {
  if constexpr (std::is_same<T, float>::value)
    if (c->imp.basis16) return run_steps<float, __half>(c, n, history);
  return run_steps<T, T>(c, n, history);
}

// Residual and assembled system of slot 0 at the current state and the given CFL, without a
// graph (bes_implicit_assemble).
template <class T>
int assemble_once(bes_ctx* c, double cfl, double* norms15) {
  ImplicitBuffers& I = c->imp;
  std::vector<int32_t> act(I.nslot, 0);
  act[0] = 1;
  std::vector<double> cf(I.nslot, cfl), P(6 * I.nslot, 0.0);
  freestream_from(&c->pinf0_host[0], c->prm.ramp_steps, c->prm.ramp_frac, I.ctl[0].host_step, &P[0]);
  IMP_TRY(c, cudaMemcpyAsync(I.act, act.data(), act.size() * 4, cudaMemcpyHostToDevice, c->stream));
  IMP_TRY(c, cudaMemcpyAsync(I.cfl_dev, cf.data(), cf.size() * 8, cudaMemcpyHostToDevice, c->stream));
  IMP_TRY(c, cudaMemcpyAsync(c->pinf_dev, P.data(), P.size() * 8, cudaMemcpyHostToDevice, c->stream));
  SlotHandles hs;
  std::memset(&hs, 0, sizeof(hs));
  enqueue_residual_all(c, c->stream, hs, 0);
  Sys<T, T> S(c);
  enqueue_assembly(S, c->stream, 0, result_norms(I.res, 0));
  IMP_TRY(c, cudaGetLastError());
  IMP_TRY(c, cudaMemcpyAsync(I.res_host.data(), I.res, sizeof(StepResult), cudaMemcpyDeviceToHost,
                             c->stream));
  int nan = 0;
  IMP_TRY(c, cudaMemcpyAsync(&nan, c->nan_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  IMP_TRY(c, cudaStreamSynchronize(c->stream));
  const double* r = I.res_host[0].norms;
  for (int v = 0; v < 5; ++v) {
    norms15[v] = r[v];
    norms15[5 + v] = r[10 + v];
    norms15[10 + v] = r[5 + v];
  }
  return check_step_nan(c, nan);
}

// True when the factorisation order is the identity and every stage is a contiguous range of
// cells in increasing order (colour order on the colour-major numbering).
inline bool colour_ranges(const SoaMesh& M) {
  if (M.n_stages < 1) return false;
  for (int64_t i = 0; i < (int64_t)M.ilu_pos.size(); ++i)
    if (M.ilu_pos[i] != i || M.stage_rows[i] != i) return false;
  return true;
}

}  // namespace

namespace bes {

void implicit_reset(bes_ctx* c) {
  for (SlotCtl& k : c->imp.ctl) {
    k = SlotCtl();
    k.cfl_actual = c->opt.courant_num;
  }
}

void implicit_release(bes_ctx* c) {
  ImplicitBuffers& I = c->imp;
  for (int p = 0; p < 2; ++p)
    for (int q = 0; q < 2; ++q)
      if (I.step_graph[p][q]) {
        cudaGraphExecDestroy(I.step_graph[p][q]);
        I.step_graph[p][q] = nullptr;
      }
  for (cudaStream_t& s : I.cap)
    if (s) {
      cudaStreamDestroy(s);
      s = nullptr;
    }
}

int implicit_allocate(bes_ctx* c) {
  ImplicitBuffers& I = c->imp;
  const bes_options& o = c->opt;
  if (o.gmres_restart < 1 || o.gmres_restart > kMaxRestart) {
    c->last_error = "GMRES_RESTART must be between 1 and 32";
    return BES_ERR_UNSUPPORTED;
  }
  if (o.precision < 0 || o.precision > 2) {
    c->last_error = "precision must be 0 (FP64 system), 1 (FP32 system) or 2 (FP32 system, "
                    "16-bit block-scaled matrix storage)";
    return BES_ERR_UNSUPPORTED;
  }
  if (o.linear_solver < 0 || o.linear_solver > 2) {
    c->last_error = "linear_solver must be 0 (block Jacobi), 1 (block ILU(0), colour order) or 2 "
                    "(block ILU(0), RCM order, level scheduled)";
    return BES_ERR_UNSUPPORTED;
  }
  if (c->nb > kMaxSlots) {
    c->last_error = "an implicit context holds at most 256 conditions";
    return BES_ERR_UNSUPPORTED;
  }
  I.prec = o.precision ? 1 : 0;
  I.packed = o.precision == 2;
  I.basis16 = I.packed;
  I.tsize = I.prec ? sizeof(float) : sizeof(double);
  I.nslot = c->nb;
  const SoaMesh& M = c->soa;
  const int64_t nc = M.nc, nf = M.nf, ns = I.nslot;
  if (o.linear_solver == 2) build_ilu_schedule(c->soa, true);
  I.use_colour_ranges = o.linear_solver == 1 && colour_ranges(c->soa);
  if (I.packed && uses_ilu(c) && !I.use_colour_ranges) {
    c->last_error = "precision 2 runs block Jacobi or the colour-ordered block ILU(0)";
    return BES_ERR_UNSUPPORTED;
  }
  I.ldv = basis_stride(nc);
  // the system in T: per condition, or one scratch shared by all (16-bit storage)
  const int64_t msl = I.packed ? 1 : ns;
  I.sA = I.packed ? 0 : 125 * nc;
  I.sDinv = I.packed ? 0 : 25 * nc;
  int rc = 0;
  rc |= imp_malloc(c, &I.A, 125 * nc * I.tsize * msl);
  rc |= imp_malloc(c, &I.Dinv, 25 * nc * I.tsize * msl);
  if (uses_ilu(c)) rc |= imp_malloc(c, &I.LU, 125 * nc * I.tsize * msl);
  if (I.packed) {
    rc |= imp_malloc(c, &I.A16, 65 * nc * sizeof(__half2) * ns);
    rc |= imp_malloc(c, (void**)&I.As, 5 * nc * sizeof(float) * ns);
    rc |= imp_malloc(c, &I.D16, 13 * nc * sizeof(__half2) * ns);
    rc |= imp_malloc(c, (void**)&I.Ds, nc * sizeof(float) * ns);
    if (uses_ilu(c)) {
      rc |= imp_malloc(c, &I.LU16, 52 * nc * sizeof(__half2) * ns);
      rc |= imp_malloc(c, (void**)&I.LUs, 4 * nc * sizeof(float) * ns);
    }
  }
  rc |= imp_malloc(c, &I.Dc, 50 * nf * I.tsize);
  rc |= imp_malloc(c, &I.b, I.ldv * I.tsize * ns);
  I.sV = (int64_t)(o.gmres_restart + 1) * I.ldv;
  rc |= imp_malloc(c, &I.V, I.sV * (I.basis16 ? sizeof(__half) : I.tsize) * ns);
  if (I.basis16) rc |= imp_malloc(c, &I.Vx, I.ldv * sizeof(float) * ns);
  rc |= imp_malloc(c, &I.Z, I.ldv * I.tsize * ns);
  rc |= imp_malloc(c, &I.W, I.ldv * I.tsize * ns);
  rc |= imp_malloc(c, &I.X, I.ldv * I.tsize * ns);
  rc |= imp_malloc(c, (void**)&I.rhs, 5 * nc * sizeof(double) * ns);
  I.red_ld = std::max<int64_t>(kRedBlocks, nblk(nc, 128));
  rc |= imp_malloc(c, (void**)&I.red, 64 * I.red_ld * sizeof(double) * ns);
  GmresDev& g = I.gm;
  rc |= imp_malloc(c, (void**)&g.H, ns * kHsize * sizeof(double));
  rc |= imp_malloc(c, (void**)&g.cs, ns * kMaxRestart * sizeof(double));
  rc |= imp_malloc(c, (void**)&g.sn, ns * kMaxRestart * sizeof(double));
  rc |= imp_malloc(c, (void**)&g.g, ns * (kMaxRestart + 1) * sizeof(double));
  rc |= imp_malloc(c, (void**)&g.y, ns * kMaxRestart * sizeof(double));
  rc |= imp_malloc(c, (void**)&g.sc, ns * 8 * sizeof(double));
  int32_t** ints[] = {&g.lin, &g.cyc, &g.jc, &g.iter, &g.second, &g.status, &g.cycles};
  for (int32_t** p : ints) rc |= imp_malloc(c, (void**)p, ns * sizeof(int32_t));
  rc |= imp_malloc(c, (void**)&g.dev, ns * kGsLd * sizeof(double));
  rc |= imp_malloc(c, (void**)&g.devf, ns * kGsLd * sizeof(float));
  rc |= imp_malloc(c, (void**)&g.counters, 3 * sizeof(unsigned long long));
  rc |= imp_malloc(c, (void**)&I.res, ns * sizeof(StepResult));
  rc |= imp_malloc(c, (void**)&I.cfl_dev, ns * sizeof(double));
  rc |= imp_malloc(c, (void**)&I.act, ns * sizeof(int32_t));
  rc |= imp_malloc(c, (void**)&I.guard_dev, sizeof(int32_t));
  rc |= imp_malloc(c, (void**)&c->prof.dev, 3 * PROF_NCAT * sizeof(unsigned long long));
  rc |= imp_malloc(c, (void**)&I.sync_count, sizeof(unsigned));
  rc |= imp_malloc(c, (void**)&I.sync_gen, sizeof(unsigned));
  rc |= imp_malloc(c, (void**)&I.sync_error, sizeof(int));
  rc |= imp_malloc(c, (void**)&I.m_own, nf);
  rc |= imp_malloc(c, (void**)&I.m_nb, nf);
  rc |= imp_malloc(c, (void**)&I.stage_rows, nc * sizeof(int32_t));
  rc |= imp_malloc(c, (void**)&I.ilu_pos, nc * sizeof(int32_t));
  if (rc) return BES_ERR_CUDA;
  IMP_TRY(c, cudaMemset(I.A, 0, 125 * nc * I.tsize * msl));  // empty slots stay zero
  IMP_TRY(c, cudaMemset(g.lin, 0, ns * sizeof(int32_t)));
  IMP_TRY(c, cudaMemset(g.cyc, 0, ns * sizeof(int32_t)));
  IMP_TRY(c, cudaMemset(g.counters, 0, 3 * sizeof(unsigned long long)));
  IMP_TRY(c, cudaMemset(I.guard_dev, 0, sizeof(int32_t)));
  IMP_TRY(c, cudaMemset(I.sync_count, 0, sizeof(unsigned)));
  IMP_TRY(c, cudaMemset(I.sync_gen, 0, sizeof(unsigned)));
  IMP_TRY(c, cudaMemset(I.sync_error, 0, sizeof(int)));
  {
    // persistent colour sweep: every block resident (occupancy x SMs), if the device can
    // launch cooperatively
    int coop = 0, sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    cudaError_t e;
    if (I.packed)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ilu_sweep_persistent_kernel<float, true>, 128, 0);
    else if (I.prec)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ilu_sweep_persistent_kernel<float, false>, 128, 0);
    else
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ilu_sweep_persistent_kernel<double, false>, 128, 0);
    I.persistent_blocks = (coop && e == cudaSuccess) ? per_sm * sms : 0;
    cudaGetLastError();
  }
  IMP_TRY(c, cudaMemset(I.res, 0, ns * sizeof(StepResult)));
  IMP_TRY(c, cudaMemset(c->prof.dev, 0, 3 * PROF_NCAT * sizeof(unsigned long long)));
  IMP_TRY(c, cudaMemcpy(I.m_own, M.f_m_own.data(), nf, cudaMemcpyHostToDevice));
  IMP_TRY(c, cudaMemcpy(I.m_nb, M.f_m_nb.data(), nf, cudaMemcpyHostToDevice));
  IMP_TRY(c, cudaMemcpy(I.stage_rows, M.stage_rows.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice));
  IMP_TRY(c, cudaMemcpy(I.ilu_pos, M.ilu_pos.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice));
  I.res_host.assign(ns, StepResult());
  I.ctl.assign(ns, SlotCtl());
  implicit_reset(c);
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
  return ctx->imp.prec ? run_steps_t<float>(ctx, n, history) : run_steps_t<double>(ctx, n, history);
}

int bes_profile(bes_ctx* ctx, int32_t enable, double* ms_out, int64_t* counts_out) {
  if (!ctx) return BES_ERR_INVALID;
  Profiler& P = ctx->prof;
  if (P.dev) {
    unsigned long long h[3 * PROF_NCAT];
    IMP_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    IMP_TRY(ctx, cudaMemcpy(h, P.dev, sizeof(h), cudaMemcpyDeviceToHost));
    IMP_TRY(ctx, cudaMemset(P.dev, 0, sizeof(h)));
    for (int k = 0; k < PROF_NCAT; ++k) {
      P.ms[k] = h[PROF_NCAT + k] * 1e-6;
      P.count[k] = (int64_t)h[2 * PROF_NCAT + k];
    }
  }
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

int bes_implicit_stats(const bes_ctx* ctx, int64_t* out) {
  if (!ctx || !out) return BES_ERR_INVALID;
  out[0] = ctx->imp.step_count;
  out[1] = ctx->imp.host_syncs;
  out[2] = (int64_t)ctx->imp.counters_host[0];
  out[3] = (int64_t)ctx->imp.counters_host[1];
  return BES_OK;
}

int bes_tuning(const bes_ctx* ctx, char* buf, size_t cap) {
  if (!ctx || !buf || cap == 0) return BES_ERR_INVALID;
  std::snprintf(buf, cap, "%s", ctx->imp.tuning.c_str());
  return BES_OK;
}

int bes_set_linear_guard(bes_ctx* ctx, int32_t max_cycles) {
  if (!ctx || max_cycles < 0) return BES_ERR_INVALID;
  if (ctx->opt.solver_type != 1 || !ctx->imp.guard_dev) return BES_ERR_INVALID;
  ctx->imp.guard = max_cycles;
  IMP_TRY(ctx, cudaMemcpyAsync(ctx->imp.guard_dev, &ctx->imp.guard, sizeof(int32_t),
                               cudaMemcpyHostToDevice, ctx->stream));
  IMP_TRY(ctx, cudaStreamSynchronize(ctx->stream));
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
  int rc = ctx->imp.prec ? assemble_once<float>(ctx, cfl, norms) : assemble_once<double>(ctx, cfl, norms);
  if (rc) return rc;
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
  return BES_OK;
}

int bes_ilu_order(bes_ctx* ctx, int64_t* order) {
  if (!ctx || !order) return BES_ERR_INVALID;
  const SoaMesh& M = ctx->soa;
  for (int64_t i = 0; i < M.nc; ++i) order[M.ilu_pos[i]] = M.cell_new2ref[i];
  return BES_OK;
}

}  // extern "C"
