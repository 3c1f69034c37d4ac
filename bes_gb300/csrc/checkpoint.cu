// Checkpoint and resume of a solve.  The reference has no restart reader (it writes output
// snapshots only, src/SolverExplicit.cpp:427-433); this keeps what a solve needs to continue
// exactly where it stopped: the FP64 state of every condition (reference numbering), each
// condition's freestream, active flag, CFL controller and step counters, and the explicit
// solver's step counter (freestream ramp).  A context resumed from a checkpoint continues bit
// for bit as the original would have.
//
// File layout (little-endian, as written by this host): magic "BESCKPT1", then int32 version
// (1), solver type, precision, conditions nb, dimension; int64 cells; int64 explicit step,
// explicit iterations done, implicit steps of the context; per condition: int32 active, 6
// doubles of freestream primitives (unramped), the implicit controller (double CFL, 5 + 5
// doubles of max residuals, int64 step count, int64 freestream-ramp step); then the state
// [nb][cells][5] doubles.
#include <cstdio>
#include <cstring>
#include <vector>

#include "context.hpp"

using namespace bes;

namespace {

constexpr char kMagic[8] = {'B', 'E', 'S', 'C', 'K', 'P', 'T', '1'};
constexpr int32_t kVersion = 1;

struct File {
  FILE* f = nullptr;
  explicit File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

template <class T>
bool put(FILE* f, const T* v, size_t n = 1) { return std::fwrite(v, sizeof(T), n, f) == n; }
template <class T>
bool get(FILE* f, T* v, size_t n = 1) { return std::fread(v, sizeof(T), n, f) == n; }

int fail(bes_ctx* c, const std::string& msg) {
  c->last_error = msg;
  return BES_ERR_INVALID;
}

}  // namespace

extern "C" int bes_checkpoint_save(bes_ctx* ctx, const char* path) {
  if (!ctx || !path) return BES_ERR_INVALID;
  const int64_t nc = ctx->soa.nc;
  const int nb = ctx->nb;
  std::vector<double> U((size_t)nb * nc * 5);
  int rc = bes_get_state(ctx, U.data());
  if (rc) return rc;
  File F(path, "wb");
  if (!F.f) return fail(ctx, std::string("cannot write checkpoint ") + path);
  const int32_t hdr[5] = {kVersion, ctx->opt.solver_type, ctx->opt.precision, nb, ctx->ref.dim};
  int64_t step_dev = 0;
  if (cudaMemcpy(&step_dev, ctx->step_dev, sizeof(step_dev), cudaMemcpyDeviceToHost) !=
      cudaSuccess)
    return fail(ctx, "cannot read the explicit step counter");
  const int64_t counters[4] = {nc, step_dev, ctx->iterations_done, ctx->imp.step_count};
  bool ok = put(F.f, kMagic, 8) && put(F.f, hdr, 5) && put(F.f, counters, 4);
  for (int k = 0; k < nb && ok; ++k) {
    const int32_t act = ctx->active_host[k];
    SlotCtl t;
    if (k < (int)ctx->imp.ctl.size()) t = ctx->imp.ctl[k];
    ok = put(F.f, &act) && put(F.f, &ctx->pinf0_host[6 * k], 6) && put(F.f, &t.cfl_actual) &&
         put(F.f, t.maxres, 5) && put(F.f, t.maxres_old, 5) && put(F.f, &t.step_count) &&
         put(F.f, &t.host_step);
  }
  ok = ok && put(F.f, U.data(), U.size());
  if (!ok) return fail(ctx, std::string("short write to checkpoint ") + path);
  return BES_OK;
}

extern "C" int bes_checkpoint_load(bes_ctx* ctx, const char* path) {
  if (!ctx || !path) return BES_ERR_INVALID;
  const int64_t nc = ctx->soa.nc;
  const int nb = ctx->nb;
  File F(path, "rb");
  if (!F.f) return fail(ctx, std::string("cannot read checkpoint ") + path);
  char magic[8];
  int32_t hdr[5];
  int64_t counters[4];
  if (!get(F.f, magic, 8) || std::memcmp(magic, kMagic, 8) != 0 || !get(F.f, hdr, 5) ||
      !get(F.f, counters, 4))
    return fail(ctx, std::string(path) + " is not a bes_gb300 checkpoint");
  if (hdr[0] != kVersion || hdr[1] != ctx->opt.solver_type || hdr[3] != nb ||
      hdr[4] != ctx->ref.dim || counters[0] != nc)
    return fail(ctx, "the checkpoint was written by a context of another solver type, "
                     "condition count or mesh");
  std::vector<int32_t> act(nb);
  std::vector<double> pinf(6 * (size_t)nb);
  std::vector<SlotCtl> ctl(nb);
  bool ok = true;
  for (int k = 0; k < nb && ok; ++k) {
    SlotCtl& t = ctl[k];
    ok = get(F.f, &act[k]) && get(F.f, &pinf[6 * k], 6) && get(F.f, &t.cfl_actual) &&
         get(F.f, t.maxres, 5) && get(F.f, t.maxres_old, 5) && get(F.f, &t.step_count) &&
         get(F.f, &t.host_step);
  }
  std::vector<double> U((size_t)nb * nc * 5);
  ok = ok && get(F.f, U.data(), U.size());
  if (!ok) return fail(ctx, std::string("short checkpoint ") + path);
  // freestream of every condition, then the state (set_condition also resets a condition's
  // controller; the saved one is restored after)
  for (int k = 0; k < nb; ++k) {
    const double mach[3] = {pinf[6 * k + 1], pinf[6 * k + 2], pinf[6 * k + 3]};
    const int rc = bes_set_condition(ctx, k, mach, U.data() + (size_t)k * nc * 5);
    if (rc) return rc;
  }
  for (int k = 0; k < nb; ++k) {
    for (int i = 0; i < 6; ++i) ctx->pinf0_host[6 * k + i] = pinf[6 * k + i];
    if (k < (int)ctx->imp.ctl.size()) ctx->imp.ctl[k] = ctl[k];
  }
  for (int i = 0; i < 6; ++i) ctx->prm.pinf[i] = ctx->pinf0_host[i];
  if (cudaMemcpy(ctx->pinf0_dev, ctx->pinf0_host.data(), 6 * (size_t)nb * sizeof(double),
                 cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(ctx->step_dev, &counters[1], sizeof(int64_t), cudaMemcpyHostToDevice) !=
          cudaSuccess)
    return fail(ctx, "cannot restore the device counters");
  ctx->host_step = counters[1];
  ctx->iterations_done = counters[2];
  ctx->imp.step_count = counters[3];
  return bes_set_active(ctx, act.data());
}
