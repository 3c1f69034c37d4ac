// Internal context shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bes_gb300.h"
#include "mesh_host.hpp"
#include "physics.cuh"

namespace bes {

// Device views passed to kernels by value.
struct DevMesh {
  int32_t nc, nf, nf_int, nf_slip, nslots, n_extra;
  const double *vol, *inv_vol, *eps2, *plen;
  const int32_t *adj, *cface, *gface;
  const double *Sc, *w, *r;
  const uint8_t* cflags;
  const int32_t* extra_cell;
  const uint8_t* extra_m;
  const int32_t *fown, *fnb, *fsrc_own, *fsrc_nb;
  const double *fn, *farea;
};

struct Params {
  GasConst gas;
  double pinf[6];        // freestream primitives (rho, u, v, w, p, T), Config.cpp:480-488
  const double* pinf_dev;  // the current step's freestream primitives (device, ramped),
                           // [6] per condition
  const double* pinf0_dev = nullptr;  // unramped freestream primitives, [6] per condition
  const int32_t* active = nullptr;    // per condition: 0 = frozen (its state is kept)
  int32_t ramp_steps;      // FREESTREAM_RAMP
  double ramp_frac;        // FREESTREAM_RAMP_START_FRAC
};

// Freestream primitives of step t (Config::getFreestreamPrimitiveVariables,
// src/Config.cpp:688-706): the velocity ramps from frac * u_inf to u_inf over ramp_steps.
BES_HD void freestream_from(const double* base, int32_t ramp_steps, double ramp_frac, int64_t t,
                            double* out) {
  for (int i = 0; i < 6; ++i) out[i] = base[i];
  if (ramp_steps > 0 && t < ramp_steps) {
    const double s = ramp_frac + (double)t / (double)ramp_steps * (1 - ramp_frac);
    for (int d = 0; d < 3; ++d) out[1 + d] = base[1 + d] * s;
  }
}
BES_HD void freestream_at(const Params& p, int64_t t, double* out) {
  freestream_from(p.pinf, p.ramp_steps, p.ramp_frac, t, out);
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
};

struct ExplicitGraph {
  cudaGraphExec_t exec = nullptr;
};

}  // namespace bes

namespace bes {
// Device-side state of restarted GMRES for every condition ("slot") of a context.  Each array
// holds one entry (or one fixed-size block) per slot; the Arnoldi loop, the Givens rotations,
// the restart decision and the convergence test run on the device (krylov_kernels.cuh).
constexpr int kMaxRestart = 32;      // GMRES_RESTART limit (Hessenberg columns)
constexpr int kHld = kMaxRestart;    // row stride of the Hessenberg matrix
constexpr int kGsLd = 128;           // Gram-Schmidt scalars per slot (see krylov_kernels.cuh)
struct GmresDev {
  double* H = nullptr;    // [slot][(kMaxRestart + 1) * kHld] rotated Hessenberg matrix
  double* cs = nullptr;   // [slot][kMaxRestart] Givens cosines
  double* sn = nullptr;   // [slot][kMaxRestart] Givens sines
  double* g = nullptr;    // [slot][kMaxRestart + 1] rotated right-hand side
  double* y = nullptr;    // [slot][kMaxRestart] least-squares solution of the cycle
  double* sc = nullptr;   // [slot][8] norm_b, eps, beta, 1/beta, |r|, rel
  int32_t* lin = nullptr;     // [slot] 1 while the slot's linear solve runs
  int32_t* cyc = nullptr;     // [slot] 1 while the slot's current restart cycle runs
  int32_t* jc = nullptr;      // [slot] Arnoldi steps done in the current cycle
  int32_t* iter = nullptr;    // [slot] Arnoldi steps done in this solve
  int32_t* second = nullptr;  // [slot] Arnoldi steps that needed a second Gram-Schmidt pass
  int32_t* status = nullptr;  // [slot] BES_OK, or BES_ERR_TIMEOUT when the cycle guard stopped it
  int32_t* cycles = nullptr;  // [slot] restart cycles of this solve
  double* dev = nullptr;      // [slot][kGsLd] Gram-Schmidt scalars (FP64)
  float* devf = nullptr;      // [slot][kGsLd] their FP32 copies
  unsigned long long* counters = nullptr;  // [3] Arnoldi, restart-cycle and second-pass bodies
                                           // executed
};

// What one implicit step reports per slot (read back once per step).
struct StepResult {
  double norms[15];  // L2[5], max[5] of the Dt/V-scaled right-hand side, L2[5] of R
  double rel;        // final relative linear residual
  int32_t iters;     // linear iterations
  int32_t second;    // of which needed a second Gram-Schmidt pass
  int32_t status;    // BES_OK or BES_ERR_TIMEOUT
  int32_t active;    // 1 if the slot took the step
};

// Host-side controller of one condition's implicit solve (CFL control, step counters).
struct SlotCtl {
  double cfl_actual = 0;
  double maxres[5] = {0, 0, 0, 0, 0};
  double maxres_old[5] = {0, 0, 0, 0, 0};
  int64_t step_count = 0;
  int64_t host_step = 0;
};

// Device buffers of the implicit path (allocated when the context is created for it).  Every
// condition of a batched context is a slot: the Krylov side (matrix copies the solver reads,
// basis, vectors, GMRES state) is per slot and the solver advances all slots together.  The
// FP32 assembly and factorisation scratch of the 16-bit storage (precision 2) is shared: the
// slots are assembled and factored one after another into it and packed into their own
// 16-bit copies.
struct ImplicitBuffers {
  int prec = 0;          // 0: FP64 system, 1: FP32 system (defect correction; precision 1 or 2)
  size_t tsize = 8;      // sizeof(T)
  int nslot = 1;
  int64_t ldv = 0;       // Krylov vector stride: 5 nc rounded up to 64 elements
  // system in T: ELL blocks [5 slots][25][nc]; per condition (precision 0/1) or one shared
  // scratch (precision 2); sA etc. are the per-condition strides in elements (0: shared)
  void* A = nullptr;
  void* LU = nullptr;    // block-ILU(0) factors in the same layout (ILU only)
  void* Dinv = nullptr;  // [25][nc] inverse diagonal (Jacobi) / inverse U_ii (ILU)
  int64_t sA = 0, sDinv = 0;
  void* Dc = nullptr;    // per-face diagonal contributions [2][25][nf] (shared)
  // Krylov side, per condition
  void* b = nullptr;     // right-hand side in T [ldv]
  void* V = nullptr;     // Krylov basis [(m+1)][ldv] (FP16 with precision 2)
  int64_t sV = 0;        // basis elements per condition
  void* Z = nullptr;     // [ldv]
  void* W = nullptr;     // [ldv]
  void* X = nullptr;     // solution dW [ldv]
  // precision 2: 16-bit block-scaled copies (half2 [slot][13][nc] + FP32 scale [slot][nc]) of
  // A (5 slots), the off-diagonal ILU factors (4 slots) and the inverse diagonal (1 slot), per
  // condition
  bool packed = false;
  void* A16 = nullptr;
  float* As = nullptr;
  void* LU16 = nullptr;
  float* LUs = nullptr;
  void* D16 = nullptr;
  float* Ds = nullptr;
  // precision 2: Krylov basis V in FP16 (kBasisScale times the value) and an FP32 copy of its
  // newest vector, the preconditioner's input
  bool basis16 = false;
  void* Vx = nullptr;
  double* rhs = nullptr;       // FP64 right-hand side [slot][5][nc]
  double* red = nullptr;       // reduction partials [slot][64][red_ld]
  int64_t red_ld = 0;
  GmresDev gm;
  StepResult* res = nullptr;   // [slot]
  std::vector<StepResult> res_host;
  double* cfl_dev = nullptr;   // [slot] CFL of the current step
  int32_t* act = nullptr;      // [slot] slots that take the current step
  int32_t* guard_dev = nullptr;  // restart-cycle limit of a linear solve (device copy)
  int32_t guard = 0;             // 0: linear_solver_max_iter + 1 cycles
  int8_t* m_own = nullptr;     // per face local index in owner / neighbour
  int8_t* m_nb = nullptr;
  int32_t* stage_rows = nullptr;  // block-ILU(0) rows grouped by stage
  int32_t* ilu_pos = nullptr;     // factorisation position of each cell
  bool use_colour_ranges = false;          // colour order on contiguous colour ranges
  // colour sweeps: one launch per colour, or one persistent launch per sweep (grid of
  // resident blocks with a bounded grid barrier between colours); chosen by the autotuner on
  // the first step unless the options fix it
  int sweep_kernel = 1;        // 1 per colour, 2 persistent, 3 per colour with loads first
  bool tuned = false;
  int persistent_blocks = 0;   // grid of the persistent sweep
  unsigned int* sync_count = nullptr;  // grid barrier: arrivals, generation, error flag
  unsigned int* sync_gen = nullptr;
  int* sync_error = nullptr;
  std::string tuning;          // the autotuner's report
  // one graph per implicit step: [profiled][snapshot], built on first use; kernel nodes of its
  // sections (top level, one slot's assembly, one Arnoldi step, one restart-cycle end)
  cudaGraphExec_t step_graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  int64_t nodes_top[2] = {0, 0}, nodes_slot[2] = {0, 0}, nodes_arn[2] = {0, 0},
          nodes_loop[2] = {0, 0}, nodes_gs2[2] = {0, 0};
  cudaStream_t cap[3] = {nullptr, nullptr, nullptr};  // streams capturing conditional bodies
  unsigned long long counters_host[3] = {0, 0, 0};
  std::vector<SlotCtl> ctl;    // [slot]
  int64_t step_count = 0;      // step calls of the context
  int64_t total_lin_iters = 0;
  int64_t gs_second_passes = 0;  // Arnoldi steps that needed a second Gram-Schmidt pass
  int64_t host_syncs = 0;        // host synchronisations inside bes_implicit_steps
  int last_iters = 0;
  double last_err = 0;
};
}  // namespace bes

namespace bes {
// Optional timing of the implicit path by kernel category (bes_profile): one-thread kernels
// read the GPU's global nanosecond timer before and after every category's work inside the
// step graph (events cannot be recorded inside its conditional nodes) and accumulate the
// elapsed time per category on the device.
enum ProfCat { PROF_RESIDUAL = 0, PROF_JACOBIAN, PROF_ASSEMBLE, PROF_ILU_FACTOR, PROF_PRECOND,
               PROF_SPMV, PROF_ORTHO, PROF_OTHER, PROF_NCAT };
struct Profiler {
  bool on = false;
  unsigned long long* dev = nullptr;  // [2 * PROF_NCAT + PROF_NCAT]: open stamp, ns, count
  double ms[PROF_NCAT] = {};
  int64_t count[PROF_NCAT] = {};
};
}  // namespace bes

struct bes_ctx {
  bes_options opt;
  bes::RefMesh ref;
  std::vector<double> nodes;  // the mesh arrays as given (the VTK writer's points and cells)
  std::vector<int64_t> tets;
  bes::SoaMesh soa;
  bes::DevMesh dm;
  bes::Params prm;
  cudaStream_t stream = nullptr;
  int device = 0;
  std::string last_error;
  std::vector<void*> allocations;  // every device allocation of the context
  // state: two snapshots (the reference's ping-pong, src/Solution.cpp:63-71)
  double* U[2] = {nullptr, nullptr};
  int cur = 0;  // snapshot holding the current state
  double* RS = nullptr;  // reconstructed face-side states [5][rs_ld]
  int64_t rs_ld = 0;
  double* FA = nullptr;  // face flux x area [5][nf]
  double* dt = nullptr;  // [nc]
  double* G = nullptr;   // optional gradient output [15][nc]
  double* PHI = nullptr; // optional limiter output [5][nc]
  double* Fface = nullptr;  // optional flux per unit area [5][nf]
  double* R = nullptr;   // optional residual [5][nc]
  // reductions
  double* partials = nullptr;  // [10][max_blocks]
  int max_blocks = 0;
  unsigned long long* dtmin = nullptr;  // global time step as ordered bits
  double* hist = nullptr;               // device history [hist_cap][10]
  int64_t hist_cap = 0;
  int64_t* iter_ctr = nullptr;
  int64_t* iter_cur = nullptr;    // history row of the running iteration
  // batched conditions (bes_create_batch): nb freestream conditions share the mesh; every
  // per-condition array holds nb copies side by side ([condition][...])
  int nb = 1;
  double* pinf0_dev = nullptr;       // [nb][6]
  int32_t* active_dev = nullptr;     // [nb]
  std::vector<double> pinf0_host;    // [nb][6]
  std::vector<int32_t> active_host;  // [nb]
  // state exchange with the caller: raw copies of [nb][nc][5] (reference numbering) into a
  // staging array, permuted and transposed on the device
  double* stage = nullptr;             // [nb][nc][5]
  int32_t* new2ref_dev = nullptr;      // [nc] device cell -> reference cell
  int* nan_flag = nullptr;  // face index + 1 of a NaN flux (0 none)
  double* pinf_dev = nullptr;     // [6] freestream primitives of the current step
  int64_t* step_dev = nullptr;    // solver step counter read by the explicit graphs
  int64_t host_step = 0;          // the same counter on the host
  // graphs: one explicit iteration for each parity of the current snapshot
  cudaGraphExec_t it_graph[2] = {nullptr, nullptr};
  // event pairs around every kernel of an explicit iteration (graph event-record nodes):
  // [stage][0/1 cell, 2/3 face, 4/5 update]
  cudaEvent_t kev[8][6] = {};
  int64_t iterations_done = 0;
  int64_t iters_since_reset = 0;  // graph launches since the history counter was reset
  bes::ImplicitBuffers imp;
  int64_t launches = 0;  // kernels launched by this context (graph nodes counted per launch)
  bes::Profiler prof;
};

namespace bes {
int check_nan_public(bes_ctx* ctx);   // synchronises; BES_ERR_NAN if a face flux was NaN
int implicit_allocate(bes_ctx* ctx);  // buffers of the implicit path
}  // namespace bes

namespace bes {
void implicit_reset(bes_ctx* c);  // a new solve: CFL control and step counters of every slot
void implicit_release(bes_ctx* c);  // graphs of the implicit path
}  // namespace bes
