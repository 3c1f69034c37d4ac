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
// Device buffers of the implicit path (allocated when the context is created for it).
struct ImplicitBuffers {
  int prec = 0;          // 0: FP64 system, 1: FP32 system (defect correction; precision 1 or 2)
  size_t tsize = 8;      // sizeof(T)
  void* A = nullptr;     // ELL blocks [5 slots][25][nc]
  void* LU = nullptr;    // block-ILU(0) factors in the same layout (ILU only)
  void* Dinv = nullptr;  // [25][nc] inverse diagonal (Jacobi) / inverse U_ii (ILU)
  void* Dc = nullptr;    // per-face diagonal contributions [2][25][nf]
  void* b = nullptr;     // right-hand side in T [5][nc]
  void* V = nullptr;     // Krylov basis [(m+1)][5 nc]
  void* Z = nullptr;     // [5 nc]
  void* W = nullptr;     // [5 nc]
  void* X = nullptr;     // solution dW [5 nc]
  // precision 2: 16-bit block-scaled copies (half2 [slot][13][nc] + FP32 scale [slot][nc]) of
  // A (5 slots), the off-diagonal ILU factors (4 slots) and the inverse diagonal (1 slot)
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
  double* rhs = nullptr;       // FP64 right-hand side [5][nc]
  double* red = nullptr;       // reduction partials [64][kRedBlocks]
  double* red_out = nullptr;   // reduced values [128]
  float* red_out_f = nullptr;  // FP32 copies of Gram-Schmidt coefficients [128]
  double* coef = nullptr;      // small coefficient vectors [64]
  int8_t* m_own = nullptr;     // per face local index in owner / neighbour
  int8_t* m_nb = nullptr;
  int32_t* stage_rows = nullptr;  // block-ILU(0) rows grouped by stage
  int32_t* ilu_pos = nullptr;     // factorisation position of each cell
  cudaGraphExec_t factor_graph = nullptr;  // ILU factorisation, all stages
  cudaGraphExec_t apply_graph = nullptr;   // ILU forward+backward sweep, in place on Z
  bool use_colour_ranges = false;          // colour order on contiguous colour ranges
  std::vector<cudaGraphExec_t> colour_graphs;  // sweeps from V_0..V_m, then from W, into Z
  double cfl_actual = 0;
  double maxres[5] = {0, 0, 0, 0, 0};
  double maxres_old[5] = {0, 0, 0, 0, 0};
  int64_t step_count = 0;
  int last_iters = 0;
  int64_t total_lin_iters = 0;
  int64_t gs_second_passes = 0;  // Arnoldi steps that needed a second Gram-Schmidt pass
  double last_err = 0;
};
}  // namespace bes

namespace bes {
// Optional event timing of the implicit path by kernel category (bes_profile).
enum ProfCat { PROF_RESIDUAL = 0, PROF_JACOBIAN, PROF_ASSEMBLE, PROF_ILU_FACTOR, PROF_PRECOND,
               PROF_SPMV, PROF_ORTHO, PROF_OTHER, PROF_NCAT };
struct Profiler {
  bool on = false;
  std::vector<cudaEvent_t> pool;                     // pairs: begin at 2k, end at 2k+1
  int next = 0;                                      // next free pair
  std::vector<std::pair<int, int>> pending;          // (category, pair)
  int open_pair[PROF_NCAT];
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
  // implicit batches step the conditions one after another through one set of implicit
  // buffers; each condition keeps its own CFL controller and step counters
  struct CondImplicit {
    double cfl_actual = 0;
    double maxres[5] = {0, 0, 0, 0, 0};
    double maxres_old[5] = {0, 0, 0, 0, 0};
    int64_t step_count = 0;
    int64_t host_step = 0;
  };
  std::vector<CondImplicit> cond_imp;  // [nb] when nb > 1
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
void prof_begin(bes_ctx* c, int cat);
void prof_end(bes_ctx* c, int cat);
void prof_collect(bes_ctx* c);  // after a synchronisation: accumulate finished pairs
}  // namespace bes
