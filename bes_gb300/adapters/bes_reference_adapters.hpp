// Adapters that put bes_gb300 behind the reference's own operator classes (joel-ho/BES), for
// a maintainer who swaps the GPU path into the reference's driver (src/BES.cpp:86-111).
// Compiled against the reference's headers (-I <reference>/include and its Eigen) and linked
// with the reference's sources and libbes_gb300.so; bes_gb300/adapters/Makefile builds them
// with bes_driver.cpp, a driver shaped like the reference's main().
//
// The reference's operators are per-face / per-cell virtual calls on CPU objects; a GPU does
// whole loops, so each adapter does one whole-mesh operation per call through the C ABI
// (include/bes_gb300.h) and keeps the result where the reference's getters read it:
//   GradientGpu            Gradient::computeGradient / getGradient  (include/Gradient.hpp:28-49)
//   LimiterGpu             Limiter::computeLimiterTerm / getLimiterValue (include/Limiter.hpp:28-51)
//   TimeStepCalculatorGpu  TimeStepCalculator::computeAllTimeStep / getTimeStep
//                          (include/TimeStepCalculator.hpp:28-46), local or global
//   FluxGpu                Flux_<double>::computeFlux (include/Flux.hpp:27-46), per face
//   SolverGpu              Solver::initialize / setUniversalInitialCondition / solve
//                          (include/Solver.hpp:70-72)
// All of them share one GpuPath: the library context built from the same .besi file and mesh.
// Errors follow the reference's convention: a message on stdout and exit(EXIT_FAILURE).
#pragma once

#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "Config.hpp"
#include "Flux.hpp"
#include "Gradient.hpp"
#include "Limiter.hpp"
#include "Mesh.hpp"
#include "SolutionSnapshot.hpp"
#include "Solver.hpp"
#include "TimeStepCalculator.hpp"
#include "bes_gb300.h"

namespace bes_ref {

// The library context of one run, built from the .besi file (options, output keys) and its
// mesh file.  State exchange with the reference's snapshots: the library keeps five
// conserved variables per cell; a 2-D snapshot has four (no spanwise momentum).
class GpuPath {
 public:
  explicit GpuPath(const std::string& besi) {
    char err[512] = {0};
    char mesh_path[1024] = {0};
    bes_options_default(&opt_);
    bes_output_default(&out_);
    if (bes_options_from_besi(besi.c_str(), &opt_, mesh_path, sizeof(mesh_path), err, sizeof(err)) ||
        bes_output_from_besi(besi.c_str(), &out_, err, sizeof(err)) ||
        bes_mesh_read_gmsh(mesh_path, &arrays_, err, sizeof(err)))
      fail(err);
    const int rc = bes_create(&arrays_, &opt_, &ctx_);
    if (rc != BES_OK) {
      std::cout << "ERROR: bes_create returned " << rc << " (" << (ctx_ ? bes_last_error(ctx_) : "")
                << "). Exiting..." << std::endl;
      exit(EXIT_FAILURE);
    }
    bes_sizes(ctx_, &nc_, &nf_);
    nvar_ = bes_mesh_dim(&arrays_) == 2 ? 4 : 5;
  }
  ~GpuPath() {
    bes_destroy(ctx_);
    bes_mesh_free(&arrays_);
  }
  GpuPath(const GpuPath&) = delete;
  GpuPath& operator=(const GpuPath&) = delete;

  bes_ctx* ctx() const { return ctx_; }
  bes_output& output() { return out_; }
  int64_t cells() const { return nc_; }
  int nvar() const { return nvar_; }
  // library variable index of the reference's variable v
  int lib_var(int v) const { return (nvar_ == 4 && v == 3) ? 4 : v; }

  void check(int rc, const char* what) const {
    if (rc == BES_OK) return;
    std::cout << "ERROR: " << what << ": " << bes_last_error(ctx_) << " Exiting..." << std::endl;
    exit(EXIT_FAILURE);
  }
  // the snapshot's conserved variables to the library (reference numbering)
  void upload(SolutionSnapshot* s) {
    std::vector<double> U(5 * nc_, 0.0);
    for (int64_t i = 0; i < nc_; ++i)
      for (int v = 0; v < nvar_; ++v)
        U[i * 5 + lib_var(v)] = s->getConservedVariable((unsigned long)i, (short)v);
    check(bes_set_state(ctx_, U.data()), "bes_set_state");
  }
  // the library's state to the snapshot
  void download(SolutionSnapshot* s) {
    std::vector<double> U(5 * nc_);
    check(bes_get_state(ctx_, U.data()), "bes_get_state");
    for (int64_t i = 0; i < nc_; ++i)
      for (int v = 0; v < nvar_; ++v)
        s->setConservedVariable((unsigned long)i, (short)v, U[i * 5 + lib_var(v)]);
  }

 private:
  static void fail(const char* err) {
    std::cout << "ERROR: " << err << " Exiting..." << std::endl;
    exit(EXIT_FAILURE);
  }
  bes_ctx* ctx_ = nullptr;
  bes_mesh_arrays arrays_{};
  bes_options opt_{};
  bes_output out_{};
  int64_t nc_ = 0, nf_ = 0;
  int nvar_ = 5;
};

// Green-Gauss gradients of the conserved variables with the slip-wall correction
// (GradientGreenGauss, src/GradientGreenGauss.cpp:21-135), on the GPU.
class GradientGpu : public Gradient {
 public:
  explicit GradientGpu(GpuPath* gpu) : gpu_(gpu) {}
  void computeGradient(SolutionSnapshot* s) override {
    if (variableType_ != CONSERVED) {
      std::cout << "ERROR: GradientGpu computes gradients of the conserved variables. Exiting..."
                << std::endl;
      exit(EXIT_FAILURE);
    }
    gpu_->upload(s);
    std::vector<double> g(15 * gpu_->cells());
    gpu_->check(bes_compute_operators(gpu_->ctx(), 1.0, nullptr, g.data(), nullptr, nullptr,
                                      nullptr, nullptr, nullptr),
                "bes_compute_operators");
    const short ndim = mesh_->getNumDim();
    for (int64_t i = 0; i < gpu_->cells(); ++i)
      for (int v = 0; v < nVariable_; ++v)
        for (int d = 0; d < ndim; ++d)
          variableGradient_[i][v][d] = g[i * 15 + gpu_->lib_var(v) * 3 + d];
  }

 private:
  GpuPath* gpu_;
};

// Venkatakrishnan limiter (LimiterVenkatakrishnan, src/LimiterVenkatakrishnan.cpp:21-128), on
// the GPU.  The library limits the gradient of the snapshot it is given, which is the gradient
// the reference passes in (computed from the same snapshot).
class LimiterGpu : public Limiter {
 public:
  explicit LimiterGpu(GpuPath* gpu) : gpu_(gpu) {}
  void computeLimiterTerm(SolutionSnapshot* s, Gradient*) override {
    gpu_->upload(s);
    std::vector<double> phi(5 * gpu_->cells());
    gpu_->check(bes_compute_operators(gpu_->ctx(), 1.0, nullptr, nullptr, phi.data(), nullptr,
                                      nullptr, nullptr, nullptr),
                "bes_compute_operators");
    for (int64_t i = 0; i < gpu_->cells(); ++i)
      for (int v = 0; v < nVariable_; ++v) gradientLimiter_[i][v] = phi[i * 5 + gpu_->lib_var(v)];
  }

 private:
  GpuPath* gpu_;
};

// Local (TimeStepCalculatorLocal, src/TimeStepCalculatorLocal.cpp:67-93) or global
// (TimeStepCalculatorGlobal, src/TimeStepCalculatorGlobal.cpp:64-98) time steps on the GPU.
class TimeStepCalculatorGpu : public TimeStepCalculator {
 public:
  TimeStepCalculatorGpu(GpuPath* gpu, bool global) : gpu_(gpu), global_(global) {}
  void initialize(Config* config, Gas* gas, Mesh* mesh) override {
    initializeBase_(config, gas, mesh);
    dt_.assign(gpu_->cells(), 0.0);
  }
  void computeAllTimeStep(SolutionSnapshot* s, const double& courantNum) override {
    gpu_->upload(s);
    gpu_->check(bes_compute_operators(gpu_->ctx(), courantNum, dt_.data(), nullptr, nullptr,
                                      nullptr, nullptr, nullptr, nullptr),
                "bes_compute_operators");
    if (global_) {
      double m = dt_.empty() ? 0.0 : dt_[0];
      for (double x : dt_) m = x < m ? x : m;
      dt_.assign(dt_.size(), m);
    }
  }
  double getTimeStep(const unsigned long& iElement) override { return dt_[iElement]; }

 private:
  GpuPath* gpu_;
  bool global_;
  std::vector<double> dt_;
};

// One face's flux (FluxRoe_ / FluxSlipWall_ / FluxFreestream_ ::computeFlux, src/FluxRoe.tpp,
// src/FluxSlipWall.tpp, src/FluxFreestream.tpp) through the per-face entry point.  A GPU
// launch per face is slow: this adapter is for checks; the solvers use whole-mesh calls.
// kind: 0 Roe, 1 slip wall, 2 freestream (the right state is the context's freestream).
class FluxGpu : public Flux_<double> {
 public:
  FluxGpu(GpuPath* gpu, int kind) : gpu_(gpu), kind_(kind) {}
  void initialize(Config* config, Gas_<double>* gas) override { initializeBase_(config, gas); }
  void computeFlux(double const* left, double const* right, double const* nHat,
                   double* flux) override {
    double UL[5] = {0, 0, 0, 0, 0}, UR[5] = {0, 0, 0, 0, 0}, n[3] = {0, 0, 0}, F[5];
    const int nv = gpu_->nvar(), nd = nv == 4 ? 2 : 3;
    for (int v = 0; v < nv; ++v) {
      UL[gpu_->lib_var(v)] = left[v];
      if (kind_ == 0) UR[gpu_->lib_var(v)] = right[v];
    }
    for (int d = 0; d < nd; ++d) n[d] = nHat[d];
    gpu_->check(bes_flux_batch(gpu_->ctx(), kind_, 1, UL, UR, n, F, nullptr, nullptr),
                "bes_flux_batch");
    for (int v = 0; v < nv; ++v) flux[v] = F[gpu_->lib_var(v)];
  }

 private:
  GpuPath* gpu_;
  int kind_;
};

// The whole solve (SolverExplicit / SolverImplicit ::solve, src/SolverExplicit.cpp:395-438,
// src/SolverImplicit.cpp:552-600) on the GPU: the same residual.csv and output files.
class SolverGpu : public Solver {
 public:
  explicit SolverGpu(GpuPath* gpu) : gpu_(gpu) {}
  void initialize(Config* config, Gas* gas, Mesh* mesh) override {
    initializeBase_(config, gas, mesh);
  }
  // the reference passes the step-0 freestream primitives (src/BES.cpp:108); the library
  // builds the same state from its options
  void setUniversalInitialCondition(double*) override {
    gpu_->check(bes_set_freestream_state(gpu_->ctx()), "bes_set_freestream_state");
  }
  void solve() override {
    gpu_->output().verbose = 1;  // the reference's console table
    gpu_->check(bes_solve(gpu_->ctx(), &gpu_->output()), "bes_solve");
  }

 private:
  GpuPath* gpu_;
};

}  // namespace bes_ref
