// Sweep scheduler of the implicit solver: a queue of freestream conditions solved to a
// residual drop through the slots of one batched context.  No counterpart in the reference,
// which solves one condition per process (src/BES.cpp:94-111, Solver::solve in
// src/SolverImplicit.cpp:552-600).  Every slot holds one condition; one implicit step
// advances all of them (one graph launch); a slot whose condition has converged (or reached
// the step limit) takes the next condition of the queue, so the batch stays full until the
// queue runs dry.
#include <chrono>
#include <cmath>
#include <vector>

#include "context.hpp"
#include "explicit_kernels.cuh"

using namespace bes;

namespace {

#define SW_TRY(ctx, call)                                                        \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      (ctx)->last_error = std::string(#call) + ": " + cudaGetErrorString(e_);    \
      return BES_ERR_CUDA;                                                       \
    }                                                                            \
  } while (0)

// State of slot k in reference numbering, U [n_cells][5].
int slot_state(bes_ctx* c, int k, double* U) {
  const int64_t nc = c->soa.nc;
  state_to_stage_kernel<<<1024, 256, 0, c->stream>>>((int)nc, 1, c->new2ref_dev,
                                                     c->U[c->cur] + (int64_t)k * 5 * nc, c->stage);
  ++c->launches;
  SW_TRY(c, cudaMemcpyAsync(U, c->stage, 5 * nc * sizeof(double), cudaMemcpyDeviceToHost,
                            c->stream));
  SW_TRY(c, cudaStreamSynchronize(c->stream));
  SW_TRY(c, cudaGetLastError());
  return BES_OK;
}

// Integrated slip-wall pressure force of a state (as bes_wall_force).
void wall_force_of(const bes_ctx* c, const double* U, double* F) {
  const RefMesh& R = c->ref;
  const double gm1 = c->prm.gas.gm1;
  F[0] = F[1] = F[2] = 0.0;
  for (int64_t f = 0; f < R.nf; ++f) {
    if (R.kind[f] != KIND_SLIP_WALL) continue;
    const double* u = &U[R.owner[f] * 5];
    const double k = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
    const double p = gm1 * (u[4] - k / (2.0 * u[0]));
    for (int d = 0; d < 3; ++d) F[d] += p * R.S[f * 3 + d];
  }
}

}  // namespace

extern "C" int bes_implicit_sweep(bes_ctx* ctx, int32_t n, const double* mach, const double* U0,
                                  const double* target, double drop, int64_t max_steps,
                                  int64_t* steps, double* final_res, double* force, double* U_out,
                                  double* seconds) {
  if (!ctx || n < 0 || !mach || max_steps < 1 || !(drop > 0.0)) return BES_ERR_INVALID;
  if (ctx->opt.solver_type != 1) {
    ctx->last_error = "bes_implicit_sweep drives the implicit solver";
    return BES_ERR_UNSUPPORTED;
  }
  typedef std::chrono::steady_clock Clock;
  const int ns = ctx->nb;
  const int64_t nc = ctx->soa.nc;
  std::vector<int> slot_cond(ns, -1);      // condition held by each slot (-1: idle)
  std::vector<double> r0(n, -1.0), last(n, 0.0);
  std::vector<int64_t> done_steps(n, 0);
  std::vector<Clock::time_point> started(n);
  std::vector<double> U(5 * nc);
  std::vector<int32_t> act(ns, 0);
  int next = 0, running = 0;
  auto load = [&](int k) -> int {
    const int q = next++;
    const int rc = bes_set_condition(ctx, k, mach + 3 * q, U0 ? U0 + (int64_t)q * nc * 5 : nullptr);
    if (rc) return rc;
    slot_cond[k] = q;
    started[q] = Clock::now();
    ++running;
    return BES_OK;
  };
  for (int k = 0; k < ns; ++k) {
    if (next < n) {
      const int rc = load(k);
      if (rc) return rc;
    }
    act[k] = slot_cond[k] >= 0;
  }
  int rc = bes_set_active(ctx, act.data());
  if (rc) return rc;
  std::vector<double> hist(19 * ns);
  while (running > 0) {
    rc = bes_implicit_steps(ctx, 1, hist.data());
    if (rc) return rc;
    bool changed = false;
    for (int k = 0; k < ns; ++k) {
      const int q = slot_cond[k];
      if (q < 0) continue;
      const double* h = &hist[19 * k];
      double r = 0.0;
      for (int v = 0; v < 5; ++v) r += h[14 + v] * h[14 + v];
      r = std::sqrt(r);
      if (r0[q] < 0) r0[q] = r;
      ++done_steps[q];
      last[q] = r0[q] > 0 ? r / r0[q] : 0.0;
      const double goal = (target && target[q] > 0) ? target[q] : drop * r0[q];
      const bool finished = r <= goal || !std::isfinite(r) || done_steps[q] >= max_steps;
      if (!finished) continue;
      // the condition is done: its results, then the slot takes the next condition
      if (seconds) seconds[q] = std::chrono::duration<double>(Clock::now() - started[q]).count();
      if (force || U_out) {
        if ((rc = slot_state(ctx, k, U.data()))) return rc;
        if (force) wall_force_of(ctx, U.data(), force + 3 * q);
        if (U_out) std::copy(U.begin(), U.end(), U_out + (int64_t)q * nc * 5);
      }
      slot_cond[k] = -1;
      --running;
      if (next < n) {
        if ((rc = load(k))) return rc;
      } else {
        act[k] = 0;
        changed = true;
      }
    }
    if (changed) {
      rc = bes_set_active(ctx, act.data());
      if (rc) return rc;
    }
  }
  for (int q = 0; q < n; ++q) {
    if (steps) steps[q] = done_steps[q];
    if (final_res) final_res[q] = last[q];
  }
  std::vector<int32_t> all(ns, 1);
  return bes_set_active(ctx, all.data());
}
