// C ABI of bes_gb300: context life cycle, state exchange, the explicit iteration as a CUDA
// graph, operator and flux entry points.  See include/bes_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>

#include "context.hpp"
#include "explicit_kernels.cuh"

using namespace bes;


namespace {

#define BES_CUDA_TRY(ctx, call)                                                      \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      (ctx)->last_error = std::string(#call) + ": " + cudaGetErrorString(e_);        \
      return BES_ERR_CUDA;                                                           \
    }                                                                                \
  } while (0)

template <class T>
int dev_alloc(bes_ctx* ctx, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    ctx->last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return BES_ERR_CUDA;
  }
  ctx->allocations.push_back(*p);
  return BES_OK;
}

template <class T>
int upload(bes_ctx* ctx, const T** dst, const std::vector<T>& src) {
  T* p = nullptr;
  int rc = dev_alloc(ctx, &p, src.size());
  if (rc) return rc;
  if (!src.empty()) BES_CUDA_TRY(ctx, cudaMemcpy(p, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  *dst = p;
  return BES_OK;
}

inline int blocks_for(int64_t n) { return (int)((n + kBlock - 1) / kBlock); }

int check_nan(bes_ctx* ctx) {
  int flag = 0;
  BES_CUDA_TRY(ctx, cudaMemcpyAsync(&flag, ctx->nan_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  BES_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (flag) {
    BES_CUDA_TRY(ctx, cudaMemsetAsync(ctx->nan_flag, 0, sizeof(int), ctx->stream));
    const int64_t f = ctx->soa.face_new2ref[flag - 1];
    char buf[256];
    std::snprintf(buf, sizeof(buf),
                  "NaN values encountered in flux across face %lld at coordinates [%e, %e, %e]",
                  (long long)f, ctx->ref.center[f * 3], ctx->ref.center[f * 3 + 1],
                  ctx->ref.center[f * 3 + 2]);
    ctx->last_error = buf;
    return BES_ERR_NAN;
  }
  return BES_OK;
}

// Enqueue one explicit multi-step iteration on ctx->stream (SolverExplicit::timeStep_), with
// an event pair around every kernel so per-kernel device times of the last iteration can be
// read back (bes_last_kernel_times).
void enqueue_iteration(bes_ctx* ctx, int cur) {
  const bes_options& o = ctx->opt;
  const DevMesh& m = ctx->dm;
  const int nb_c = blocks_for(m.nc), nb_f = blocks_for(m.nf);
  const dim3 gc(nb_c, ctx->nb), gf(nb_f, ctx->nb);  // y: condition
  double* Un = ctx->U[cur];
  double* Uk = ctx->U[cur ^ 1];
  const int local = o.local_time_step;
  cudaStream_t s = ctx->stream;
  freestream_step_kernel<<<1, 128, 0, s>>>(ctx->prm, ctx->nb, ctx->step_dev, ctx->pinf_dev,
                                           ctx->dtmin, ctx->iter_ctr, ctx->iter_cur);
  for (int k = 0; k < o.n_stage; ++k) {
    cudaEvent_t* e = ctx->kev[k];
    const double* Uin = (k == 0) ? Un : Uk;
    cudaEventRecordWithFlags(e[0], s, cudaEventRecordExternal);
    if (k == 0)
      cell_recon_kernel<true, false><<<gc, kBlock, 0, s>>>(
          m, ctx->prm, Uin, ctx->RS, ctx->rs_ld, ctx->dt, o.courant_num, local, ctx->dtmin,
          nullptr, nullptr);
    else
      cell_recon_kernel<false, false><<<gc, kBlock, 0, s>>>(
          m, ctx->prm, Uin, ctx->RS, ctx->rs_ld, ctx->dt, o.courant_num, local, ctx->dtmin,
          nullptr, nullptr);
    cudaEventRecordWithFlags(e[1], s, cudaEventRecordExternal);
    cudaEventRecordWithFlags(e[2], s, cudaEventRecordExternal);
    face_flux_kernel<false><<<gf, kBlock, 0, s>>>(m, ctx->prm, ctx->RS, ctx->rs_ld, ctx->FA,
                                                  nullptr, ctx->nan_flag);
    cudaEventRecordWithFlags(e[3], s, cudaEventRecordExternal);
    cudaEventRecordWithFlags(e[4], s, cudaEventRecordExternal);
    if (k == o.n_stage - 1)
      update_kernel<true><<<gc, kBlock, 0, s>>>(m, ctx->FA, Un, Uk, ctx->dt, ctx->dtmin, local,
                                                o.stage_coeff[k], ctx->partials, nullptr,
                                                ctx->prm.active);
    else
      update_kernel<false><<<gc, kBlock, 0, s>>>(m, ctx->FA, Un, Uk, ctx->dt, ctx->dtmin, local,
                                                 o.stage_coeff[k], ctx->partials, nullptr,
                                                 ctx->prm.active);
    cudaEventRecordWithFlags(e[5], s, cudaEventRecordExternal);
  }
  finalize_norms_kernel<<<ctx->nb, kBlock, 0, s>>>(ctx->partials, nb_c, ctx->hist, ctx->hist_cap,
                                                   ctx->iter_cur);
}

int build_graphs(bes_ctx* ctx) {
  for (int k = 0; k < 8; ++k)
    for (int q = 0; q < 6; ++q) BES_CUDA_TRY(ctx, cudaEventCreate(&ctx->kev[k][q]));
  for (int cur = 0; cur < 2; ++cur) {
    cudaGraph_t g;
    BES_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_iteration(ctx, cur);
    BES_CUDA_TRY(ctx, cudaStreamEndCapture(ctx->stream, &g));
    BES_CUDA_TRY(ctx, cudaGraphInstantiate(&ctx->it_graph[cur], g, 0));
    cudaGraphDestroy(g);
  }
  return BES_OK;
}

int create_context(const bes_mesh_arrays* mesh, const bes_options* opt, int n_cond,
                   const double* mach, bes_ctx** out);

}  // namespace

namespace bes {
int check_nan_public(bes_ctx* ctx) { return check_nan(ctx); }
}  // namespace bes

extern "C" {

const char* bes_build_info(void) { return "bes_gb300 sm_103a fp64"; }

void bes_options_default(bes_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->solver_type = 0;
  o->local_time_step = 0;
  o->n_stage = 4;
  o->muscl_face_vector = 0;
  o->stage_coeff[0] = 0.0833;
  o->stage_coeff[1] = 0.2069;
  o->stage_coeff[2] = 0.4265;
  o->stage_coeff[3] = 1.0;
  o->courant_num = 2.0;
  o->adaptive_courant_num_max = 0.0;
  o->adaptive_courant_num_exponent[0] = 1.0;
  o->adaptive_courant_num_exponent[1] = 1.0;
  o->venkatakrishnan_factor = 5.0;
  o->harten_correction_limit = 0.05;
  o->gas_constant = 287.0;
  o->specific_heat_ratio = 1.4;
  o->number_of_time_step = 0;
  o->linear_solver = 0;
  o->linear_solver_max_iter = 1000;
  o->gmres_restart = 30;
  o->linear_solver_tol = 1e-7;
  o->jacobian_repeat = 0;  // the reference's: once per conserved variable of the mesh
  o->precision = 0;
  o->cfl_ramp_steps = 0;
}

int bes_create(const bes_mesh_arrays* mesh, const bes_options* opt, bes_ctx** out) {
  if (!opt) return BES_ERR_INVALID;
  return create_context(mesh, opt, 1, opt->freestream_mach, out);
}

int bes_create_batch(const bes_mesh_arrays* mesh, const bes_options* opt, int32_t n_cond,
                     const double* mach, bes_ctx** out) {
  if (!opt || !mach || n_cond < 1) return BES_ERR_INVALID;
  return create_context(mesh, opt, n_cond, mach, out);
}

}  // extern "C"

namespace {

int create_context(const bes_mesh_arrays* mesh, const bes_options* opt, int n_cond,
                   const double* mach, bes_ctx** out) {
  if (!mesh || !opt || !out) return BES_ERR_INVALID;
  *out = nullptr;
  if (opt->n_stage < 1 || opt->n_stage > 8) return BES_ERR_INVALID;
  std::unique_ptr<bes_ctx> ctx(new (std::nothrow) bes_ctx());
  if (!ctx) return BES_ERR_INVALID;
  ctx->opt = *opt;
  ctx->nb = n_cond;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    *out = nullptr;
    return BES_ERR_CUDA;
  }
  cudaGetDevice(&ctx->device);
  std::string err;
  if (!build_ref_mesh(mesh->nodes, mesh->n_nodes, mesh->btris, mesh->btags, mesh->n_btris,
                      mesh->tets, mesh->n_tets, bes_mesh_dim(mesh), opt->muscl_face_vector != 0,
                      ctx->ref, err)) {
    return BES_ERR_MESH;
  }
  // Q9: the reference adds every Jacobian block once per conserved variable (its addToBlock
  // sits inside the loop over the variables, src/SolverImplicit.cpp:425-455, 465-502): five
  // times in 3-D, four times in 2-D
  if (ctx->opt.jacobian_repeat <= 0) ctx->opt.jacobian_repeat = ctx->ref.dim == 2 ? 4 : 5;
  build_soa(ctx->ref, opt->venkatakrishnan_factor, opt->muscl_face_vector != 0, true, ctx->soa);
  ctx->nodes.assign(mesh->nodes, mesh->nodes + mesh->n_nodes * 3);
  ctx->tets.assign(mesh->tets, mesh->tets + mesh->n_tets * (bes_mesh_dim(mesh) + 1));
  const SoaMesh& S = ctx->soa;
  bes_ctx* c = ctx.get();
  BES_CUDA_TRY(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  DevMesh& m = c->dm;
  m.nc = S.nc;
  m.nf = S.nf;
  m.nf_int = S.nf_int;
  m.nf_slip = S.nf_slip;
  m.nslots = S.nslots;
  m.n_extra = S.n_extra;
  int rc = 0;
  rc |= upload(c, &m.vol, S.vol);
  rc |= upload(c, &m.inv_vol, S.inv_vol);
  rc |= upload(c, &m.eps2, S.eps2);
  rc |= upload(c, &m.plen, S.plen);
  rc |= upload(c, &m.adj, S.adj);
  rc |= upload(c, &m.cface, S.cface);
  rc |= upload(c, &m.gface, S.gface);
  rc |= upload(c, &m.Sc, S.Sc);
  rc |= upload(c, &m.w, S.w);
  rc |= upload(c, &m.r, S.r);
  rc |= upload(c, &m.cflags, S.cflags);
  rc |= upload(c, &m.extra_cell, S.extra_cell);
  rc |= upload(c, &m.extra_m, S.extra_m);
  rc |= upload(c, &m.fown, S.fown);
  rc |= upload(c, &m.fnb, S.fnb);
  rc |= upload(c, &m.fsrc_own, S.fsrc_own);
  rc |= upload(c, &m.fsrc_nb, S.fsrc_nb);
  rc |= upload(c, &m.fn, S.fn);
  rc |= upload(c, &m.farea, S.farea);
  if (rc) return BES_ERR_CUDA;
  const int64_t nc = S.nc, nf = S.nf, nb = n_cond;
  c->rs_ld = nc * S.nslots + S.n_extra;
  rc |= dev_alloc(c, &c->U[0], 5 * nc * nb);
  rc |= dev_alloc(c, &c->U[1], 5 * nc * nb);
  rc |= dev_alloc(c, &c->RS, 5 * c->rs_ld * nb);
  rc |= dev_alloc(c, &c->FA, 5 * nf * nb);
  rc |= dev_alloc(c, &c->dt, nc * nb);
  c->max_blocks = blocks_for(nc);
  rc |= dev_alloc(c, &c->partials, 10 * (size_t)c->max_blocks * nb);
  rc |= dev_alloc(c, &c->dtmin, nb);
  c->hist_cap = std::max<int64_t>(16, 4096 / nb);  // iterations per history chunk
  rc |= dev_alloc(c, &c->hist, 10 * c->hist_cap * nb);
  rc |= dev_alloc(c, &c->iter_ctr, 1);
  rc |= dev_alloc(c, &c->iter_cur, 1);
  rc |= dev_alloc(c, &c->nan_flag, 1);
  rc |= dev_alloc(c, &c->pinf_dev, 6 * nb);
  rc |= dev_alloc(c, &c->pinf0_dev, 6 * nb);
  rc |= dev_alloc(c, &c->active_dev, nb);
  rc |= dev_alloc(c, &c->step_dev, 1);
  rc |= dev_alloc(c, &c->stage, 5 * nc * nb);
  rc |= dev_alloc(c, &c->new2ref_dev, nc);
  if (rc) return BES_ERR_CUDA;
  {
    std::vector<int32_t> n2r(nc);
    for (int64_t i = 0; i < nc; ++i) n2r[i] = (int32_t)S.cell_new2ref[i];
    BES_CUDA_TRY(c, cudaMemcpy(c->new2ref_dev, n2r.data(), nc * sizeof(int32_t),
                               cudaMemcpyHostToDevice));
  }
  BES_CUDA_TRY(c, cudaMemset(c->iter_ctr, 0, sizeof(int64_t)));
  BES_CUDA_TRY(c, cudaMemset(c->nan_flag, 0, sizeof(int)));
  // gas and freestream (Config::initializePostMesh, src/Config.cpp:480-488), per condition
  c->prm.gas = make_gas(opt->gas_constant, opt->specific_heat_ratio, opt->harten_correction_limit);
  c->pinf0_host.assign(6 * nb, 0.0);
  const int S_dim = c->ref.dim;
  for (int64_t b = 0; b < nb; ++b) {
    double* p = &c->pinf0_host[6 * b];
    p[0] = 1.0;
    // a 2-D mesh reads the first two FREESTREAM_MACH components (velocity w stays 0)
    for (int d = 0; d < S_dim; ++d) p[1 + d] = mach[3 * b + d];
    p[4] = 1.0 / opt->specific_heat_ratio;
    p[5] = 1.0 / (opt->specific_heat_ratio * opt->gas_constant);
  }
  for (int i = 0; i < 6; ++i) c->prm.pinf[i] = c->pinf0_host[i];
  BES_CUDA_TRY(c, cudaMemcpy(c->pinf0_dev, c->pinf0_host.data(), 6 * nb * sizeof(double),
                             cudaMemcpyHostToDevice));
  c->active_host.assign(nb, 1);
  BES_CUDA_TRY(c, cudaMemcpy(c->active_dev, c->active_host.data(), nb * sizeof(int32_t),
                             cudaMemcpyHostToDevice));
  c->prm.pinf_dev = c->pinf_dev;
  c->prm.pinf0_dev = c->pinf0_dev;
  c->prm.active = nb > 1 ? c->active_dev : nullptr;
  c->prm.ramp_steps = opt->freestream_ramp;
  c->prm.ramp_frac = opt->freestream_ramp_start_frac;
  rc = build_graphs(c);
  if (rc) return rc;
  if (opt->solver_type == 1) {
    rc = implicit_allocate(c);
    if (rc) return rc;
  }
  rc = bes_set_freestream_state(c);
  if (rc) return rc;
  *out = ctx.release();
  return BES_OK;
}

}  // namespace

extern "C" {

void bes_destroy(bes_ctx* ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (int i = 0; i < 2; ++i)
    if (ctx->it_graph[i]) cudaGraphExecDestroy(ctx->it_graph[i]);
  for (int k = 0; k < 8; ++k)
    for (int q = 0; q < 6; ++q)
      if (ctx->kev[k][q]) cudaEventDestroy(ctx->kev[k][q]);
  implicit_release(ctx);
  for (void* p : ctx->allocations) cudaFree(p);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* bes_last_error(const bes_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int bes_sizes(const bes_ctx* ctx, int64_t* n_cells, int64_t* n_faces) {
  if (!ctx) return BES_ERR_INVALID;
  if (n_cells) *n_cells = ctx->soa.nc;
  if (n_faces) *n_faces = ctx->soa.nf;
  return BES_OK;
}

int bes_set_freestream_state(bes_ctx* ctx) {
  if (!ctx) return BES_ERR_INVALID;
  // A new solve: step counter, CFL control and freestream ramp restart at step 0.
  ctx->host_step = 0;
  implicit_reset(ctx);
  const int64_t zero = 0;
  BES_CUDA_TRY(ctx, cudaMemcpy(ctx->step_dev, &zero, sizeof(zero), cudaMemcpyHostToDevice));
  // GasPerfect_::computeAllConservedVariable of the step-0 freestream primitives
  // (:182-216; setUniversalInitialCondition gets getFreestreamPrimitiveVariables(0)), for
  // every condition
  const int64_t nc = ctx->soa.nc, nb = ctx->nb;
  std::vector<double> soa(5 * nc * nb), P(6 * nb);
  for (int64_t b = 0; b < nb; ++b) {
    double* p = &P[6 * b];
    freestream_from(&ctx->pinf0_host[6 * b], ctx->prm.ramp_steps, ctx->prm.ramp_frac, 0, p);
    double Uf[5];
    Uf[0] = p[0];
    double s = 0;
    for (int d = 0; d < 3; ++d) {
      Uf[1 + d] = Uf[0] * p[1 + d];
      s += p[1 + d] * p[1 + d];
    }
    Uf[4] = Uf[0] * (ctx->prm.gas.cv * p[5] + s / 2.0);
    for (int v = 0; v < 5; ++v)
      std::fill(soa.begin() + (b * 5 + v) * nc, soa.begin() + (b * 5 + v + 1) * nc, Uf[v]);
  }
  BES_CUDA_TRY(ctx, cudaMemcpy(ctx->pinf_dev, P.data(), P.size() * sizeof(double),
                               cudaMemcpyHostToDevice));
  ctx->cur = 0;
  BES_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->U[0], soa.data(), soa.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  BES_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return BES_OK;
}

int bes_set_state(bes_ctx* ctx, const double* U) {
  if (!ctx || !U) return BES_ERR_INVALID;
  const int64_t nc = ctx->soa.nc, nb = ctx->nb;
  BES_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->stage, U, (size_t)nb * nc * 5 * sizeof(double),
                                    cudaMemcpyHostToDevice, ctx->stream));
  state_from_stage_kernel<<<1024, 256, 0, ctx->stream>>>((int)nc, (int)nb, ctx->new2ref_dev,
                                                         ctx->stage, ctx->U[ctx->cur]);
  ++ctx->launches;
  BES_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  BES_CUDA_TRY(ctx, cudaGetLastError());
  return BES_OK;
}

int bes_get_state(bes_ctx* ctx, double* U) {
  if (!ctx || !U) return BES_ERR_INVALID;
  const int64_t nc = ctx->soa.nc, nb = ctx->nb;
  state_to_stage_kernel<<<1024, 256, 0, ctx->stream>>>((int)nc, (int)nb, ctx->new2ref_dev,
                                                       ctx->U[ctx->cur], ctx->stage);
  ++ctx->launches;
  BES_CUDA_TRY(ctx, cudaMemcpyAsync(U, ctx->stage, (size_t)nb * nc * 5 * sizeof(double),
                                    cudaMemcpyDeviceToHost, ctx->stream));
  BES_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  BES_CUDA_TRY(ctx, cudaGetLastError());
  return BES_OK;
}

int bes_explicit_iterations(bes_ctx* ctx, int64_t n, double* history) {
  if (!ctx || n < 0) return BES_ERR_INVALID;
  if (ctx->opt.solver_type != 0) {
    ctx->last_error = "context was created for the implicit solver";
    return BES_ERR_INVALID;
  }
  int64_t done = 0;
  while (done < n) {
    const int64_t chunk = std::min<int64_t>(n - done, ctx->hist_cap);
    BES_CUDA_TRY(ctx, cudaMemsetAsync(ctx->iter_ctr, 0, sizeof(int64_t), ctx->stream));
    ctx->iters_since_reset = 0;
    int rc = bes_explicit_enqueue(ctx, chunk);
    if (rc) return rc;
    if (history)
      BES_CUDA_TRY(ctx, cudaMemcpyAsync(history + done * 10 * ctx->nb, ctx->hist,
                                        chunk * 10 * ctx->nb * sizeof(double),
                                        cudaMemcpyDeviceToHost, ctx->stream));
    rc = check_nan(ctx);  // synchronises the stream
    if (rc) return rc;
    done += chunk;
  }
  return BES_OK;
}

int bes_compute_operators(bes_ctx* ctx, double cfl, double* dt, double* grad, double* limiter,
                          double* face_UL, double* face_UR, double* face_flux, double* residual) {
  if (!ctx) return BES_ERR_INVALID;
  if (ctx->nb != 1) {
    ctx->last_error = "operators are evaluated on single-condition contexts";
    return BES_ERR_UNSUPPORTED;
  }
  bes_ctx* c = ctx;
  const int64_t nc = c->soa.nc, nf = c->soa.nf;
  if (!c->G) {
    int rc = 0;
    rc |= dev_alloc(c, &c->G, 15 * nc);
    rc |= dev_alloc(c, &c->PHI, 5 * nc);
    rc |= dev_alloc(c, &c->Fface, 5 * nf);
    rc |= dev_alloc(c, &c->R, 5 * nc);
    if (rc) return BES_ERR_CUDA;
  }
  const DevMesh& m = c->dm;
  double* Ucur = c->U[c->cur];
  double* scratch = c->U[c->cur ^ 1];
  double P[6];
  freestream_at(c->prm, c->host_step, P);
  BES_CUDA_TRY(c, cudaMemcpyAsync(c->pinf_dev, P, sizeof(P), cudaMemcpyHostToDevice, c->stream));
  reset_dtmin_kernel<<<1, 1, 0, c->stream>>>(c->dtmin);
  cell_recon_kernel<true, true><<<blocks_for(nc), kBlock, 0, c->stream>>>(
      m, c->prm, Ucur, c->RS, c->rs_ld, c->dt, cfl, 1, c->dtmin, c->G, c->PHI);
  face_flux_kernel<true><<<blocks_for(nf), kBlock, 0, c->stream>>>(m, c->prm, c->RS, c->rs_ld,
                                                                   c->FA, c->Fface, c->nan_flag);
  update_kernel<false><<<blocks_for(nc), kBlock, 0, c->stream>>>(
      m, c->FA, Ucur, scratch, c->dt, c->dtmin, 1, 0.0, c->partials, c->R);
  BES_CUDA_TRY(c, cudaGetLastError());
  BES_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  auto fetch = [&](const double* d, int64_t count) {
    std::vector<double> h(count);
    cudaMemcpy(h.data(), d, count * 8, cudaMemcpyDeviceToHost);
    return h;
  };
  if (dt) {
    auto h = fetch(c->dt, nc);
    for (int64_t i = 0; i < nc; ++i) dt[c->soa.cell_new2ref[i]] = h[i];
  }
  if (grad) {
    auto h = fetch(c->G, 15 * nc);
    for (int64_t i = 0; i < nc; ++i)
      for (int q = 0; q < 15; ++q) grad[c->soa.cell_new2ref[i] * 15 + q] = h[q * nc + i];
  }
  if (limiter) {
    auto h = fetch(c->PHI, 5 * nc);
    for (int64_t i = 0; i < nc; ++i)
      for (int v = 0; v < 5; ++v) limiter[c->soa.cell_new2ref[i] * 5 + v] = h[v * nc + i];
  }
  if (face_UL || face_UR) {
    auto h = fetch(c->RS, 5 * c->rs_ld);
    for (int64_t j = 0; j < nf; ++j) {
      const int64_t f = c->soa.face_new2ref[j];
      for (int v = 0; v < 5; ++v) {
        if (face_UL) face_UL[f * 5 + v] = h[v * c->rs_ld + c->soa.fsrc_own[j]];
        if (face_UR) face_UR[f * 5 + v] = c->soa.fsrc_nb[j] >= 0 ? h[v * c->rs_ld + c->soa.fsrc_nb[j]] : 0.0;
      }
    }
  }
  if (face_flux) {
    auto h = fetch(c->Fface, 5 * nf);
    for (int64_t j = 0; j < nf; ++j)
      for (int v = 0; v < 5; ++v) face_flux[c->soa.face_new2ref[j] * 5 + v] = h[v * nf + j];
  }
  if (residual) {
    auto h = fetch(c->R, 5 * nc);
    for (int64_t i = 0; i < nc; ++i)
      for (int v = 0; v < 5; ++v) residual[c->soa.cell_new2ref[i] * 5 + v] = h[v * nc + i];
  }
  return check_nan(c);
}

int bes_explicit_enqueue(bes_ctx* ctx, int64_t n) {
  if (!ctx || n < 0) return BES_ERR_INVALID;
  if (ctx->opt.solver_type != 0) return BES_ERR_INVALID;
  for (int64_t i = 0; i < n; ++i) {
    if (ctx->iters_since_reset >= ctx->hist_cap) {
      BES_CUDA_TRY(ctx, cudaMemsetAsync(ctx->iter_ctr, 0, sizeof(int64_t), ctx->stream));
      ctx->iters_since_reset = 0;
    }
    BES_CUDA_TRY(ctx, cudaGraphLaunch(ctx->it_graph[ctx->cur], ctx->stream));
    ctx->launches += 2 + 3 * ctx->opt.n_stage;  // kernel nodes of one iteration graph
    ++ctx->host_step;
    ctx->cur ^= 1;
    ++ctx->iters_since_reset;
  }
  ctx->iterations_done += n;
  return BES_OK;
}

int bes_synchronize(bes_ctx* ctx) {
  if (!ctx) return BES_ERR_INVALID;
  BES_CUDA_TRY(ctx, cudaGetLastError());
  return check_nan(ctx);
}

void* bes_stream(bes_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int bes_last_kernel_times(bes_ctx* ctx, double* ms_out) {
  if (!ctx || !ms_out) return BES_ERR_INVALID;
  BES_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  double acc[3] = {0, 0, 0};
  for (int k = 0; k < ctx->opt.n_stage; ++k)
    for (int q = 0; q < 3; ++q) {
      float ms = 0;
      BES_CUDA_TRY(ctx, cudaEventElapsedTime(&ms, ctx->kev[k][2 * q], ctx->kev[k][2 * q + 1]));
      acc[q] += ms;
    }
  ms_out[0] = acc[0];
  ms_out[1] = acc[1];
  ms_out[2] = acc[2];
  ms_out[3] = acc[0] + acc[1] + acc[2];
  return BES_OK;
}

int bes_counters(const bes_ctx* ctx, int64_t* out) {
  if (!ctx || !out) return BES_ERR_INVALID;
  out[0] = ctx->launches;
  out[1] = ctx->iterations_done;
  out[2] = ctx->imp.step_count;
  out[3] = ctx->imp.total_lin_iters;
  out[4] = ctx->imp.gs_second_passes;
  return BES_OK;
}

int bes_wall_force(bes_ctx* ctx, double* force) {
  if (!ctx || !force) return BES_ERR_INVALID;
  // Integrated slip-wall pressure force sum_f p_owner S_f with the owner cell's pressure, the
  // quantity of the reference's slip-wall output (SolutionSnapshot::writeSlipWallToCsv,
  // src/SolutionSnapshot.cpp:268-309), in non-dimensional units, summed in face order.
  // Batched contexts: force [n_cond][3].
  const int64_t nc = ctx->soa.nc;
  std::vector<double> U(5 * nc * ctx->nb);
  int rc = bes_get_state(ctx, U.data());
  if (rc) return rc;
  const RefMesh& R = ctx->ref;
  const double gm1 = ctx->prm.gas.gm1;
  for (int64_t b = 0; b < ctx->nb; ++b) {
    double F[3] = {0, 0, 0};
    for (int64_t f = 0; f < R.nf; ++f) {
      if (R.kind[f] != KIND_SLIP_WALL) continue;
      const double* u = &U[(b * nc + R.owner[f]) * 5];
      const double k = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
      const double p = gm1 * (u[4] - k / (2.0 * u[0]));
      for (int d = 0; d < 3; ++d) F[d] += p * R.S[f * 3 + d];
    }
    for (int d = 0; d < 3; ++d) force[b * 3 + d] = F[d];
  }
  return BES_OK;
}

int bes_conditions(const bes_ctx* ctx, int32_t* n_cond) {
  if (!ctx || !n_cond) return BES_ERR_INVALID;
  *n_cond = ctx->nb;
  return BES_OK;
}

int bes_set_active(bes_ctx* ctx, const int32_t* active) {
  if (!ctx || !active) return BES_ERR_INVALID;
  for (int b = 0; b < ctx->nb; ++b) ctx->active_host[b] = active[b] ? 1 : 0;
  BES_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->active_dev, ctx->active_host.data(),
                                    ctx->nb * sizeof(int32_t), cudaMemcpyHostToDevice,
                                    ctx->stream));
  BES_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return BES_OK;
}

int bes_set_condition(bes_ctx* ctx, int32_t cond, const double* mach, const double* U) {
  if (!ctx || cond < 0 || cond >= ctx->nb) return BES_ERR_INVALID;
  const int64_t nc = ctx->soa.nc;
  double* p = &ctx->pinf0_host[6 * cond];
  if (mach) {
    p[0] = 1.0;
    for (int d = 0; d < 3; ++d) p[1 + d] = d < ctx->ref.dim ? mach[d] : 0.0;
    p[4] = 1.0 / ctx->opt.specific_heat_ratio;
    p[5] = 1.0 / (ctx->opt.specific_heat_ratio * ctx->opt.gas_constant);
    if (cond == 0)
      for (int i = 0; i < 6; ++i) ctx->prm.pinf[i] = p[i];
    BES_CUDA_TRY(ctx, cudaMemcpy(ctx->pinf0_dev + 6 * cond, p, 6 * sizeof(double),
                                 cudaMemcpyHostToDevice));
  }
  // the condition's state in reference numbering, or its step-0 freestream
  std::vector<double> Uh(5 * nc);
  if (U) {
    std::copy(U, U + 5 * nc, Uh.begin());
  } else {
    double q[6];
    freestream_from(p, ctx->prm.ramp_steps, ctx->prm.ramp_frac, 0, q);
    double Uf[5];
    Uf[0] = q[0];
    double k2 = 0;
    for (int d = 0; d < 3; ++d) {
      Uf[1 + d] = Uf[0] * q[1 + d];
      k2 += q[1 + d] * q[1 + d];
    }
    Uf[4] = Uf[0] * (ctx->prm.gas.cv * q[5] + k2 / 2.0);
    for (int64_t i = 0; i < nc; ++i)
      for (int v = 0; v < 5; ++v) Uh[i * 5 + v] = Uf[v];
  }
  BES_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->stage, Uh.data(), 5 * nc * sizeof(double),
                                    cudaMemcpyHostToDevice, ctx->stream));
  state_from_stage_kernel<<<1024, 256, 0, ctx->stream>>>(
      (int)nc, 1, ctx->new2ref_dev, ctx->stage, ctx->U[ctx->cur] + (int64_t)cond * 5 * nc);
  ++ctx->launches;
  if (cond < (int)ctx->imp.ctl.size()) {
    ctx->imp.ctl[cond] = SlotCtl();
    ctx->imp.ctl[cond].cfl_actual = ctx->opt.courant_num;
  }
  ctx->active_host[cond] = 1;
  BES_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->active_dev, ctx->active_host.data(),
                                    ctx->nb * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
  BES_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  BES_CUDA_TRY(ctx, cudaGetLastError());
  return BES_OK;
}

int bes_sweep_run(bes_ctx* ctx, int64_t max_iter, double drop, int64_t check_every,
                  int64_t* iters, double* final_drop) {
  if (!ctx || max_iter < 0 || check_every < 1) return BES_ERR_INVALID;
  if (ctx->opt.solver_type != 0) {
    ctx->last_error = "bes_sweep_run drives the explicit solver";
    return BES_ERR_UNSUPPORTED;
  }
  const int nb = ctx->nb;
  std::vector<double> r0(nb, -1.0), last(nb, 0.0);
  std::vector<int64_t> conv(nb, -1);
  std::vector<int32_t> act(nb, 1);
  int rc = bes_set_active(ctx, act.data());
  if (rc) return rc;
  std::vector<double> hist;
  int64_t done = 0;
  int n_active = nb;
  while (done < max_iter && n_active > 0) {
    const int64_t n = std::min<int64_t>(check_every, max_iter - done);
    hist.assign((size_t)n * nb * 10, 0.0);
    rc = bes_explicit_iterations(ctx, n, hist.data());
    if (rc) return rc;
    for (int64_t q = 0; q < n; ++q)
      for (int b = 0; b < nb; ++b) {
        if (!act[b] || conv[b] >= 0) continue;
        const double* h = &hist[((size_t)q * nb + b) * 10];
        double r = 0.0;
        for (int v = 0; v < 5; ++v) r += h[v] * h[v];
        r = std::sqrt(r);
        if (r0[b] < 0) r0[b] = r;
        last[b] = r0[b] > 0 ? r / r0[b] : 0.0;
        if (!(r <= drop * r0[b]) && std::isfinite(r)) continue;
        conv[b] = done + q + 1;  // converged (or diverged to a non-finite residual)
      }
    done += n;
    bool changed = false;
    for (int b = 0; b < nb; ++b)
      if (act[b] && conv[b] >= 0) {
        act[b] = 0;
        --n_active;
        changed = true;
      }
    if (changed && n_active > 0) {
      rc = bes_set_active(ctx, act.data());
      if (rc) return rc;
    }
  }
  for (int b = 0; b < nb; ++b) {
    if (iters) iters[b] = conv[b] >= 0 ? conv[b] : done;
    if (final_drop) final_drop[b] = last[b];
  }
  std::fill(act.begin(), act.end(), 1);
  return bes_set_active(ctx, act.data());
}

}  // extern "C"
