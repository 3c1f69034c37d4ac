// Driver for the patched reference build (joel-ho/BES compiled from its own sources).
// TEST INFRASTRUCTURE ONLY: it runs the reference's own objects and dumps FP64 binary data
// that pins the CPU restatement in oracle/ (the reference's ASCII outputs carry ~6 digits).
//
//   bes_ref_harness <case.besi> <outdir> <n_steps> [explicit|implicit|kat] [dump_ops] [write]
//                   [geometry]
//
// It builds Config, Mesh, Gas and the solver exactly as main() does (src/BES.cpp:86-108),
// sets the freestream initial condition, then calls the solver's own timeStep_ n_steps
// times.  After each step it records norms of the residual the reference logs:
//   explicit: R of the last multi-step stage (subResidual_, src/SolverExplicit.cpp:326-362);
//   implicit: the Dt/V-scaled right-hand side explicitFlux_ (src/SolverImplicit.cpp:519-523)
// plus the linear-solver iterations/error and the CFL.  With dump_ops it also writes, for
// the initial state, the geometry, the time steps, Green-Gauss gradients, Venkatakrishnan
// limiters, per-face MUSCL states and fluxes, first-order flux Jacobians and (implicit) the
// assembled matrix and right-hand side.  With write it finally calls the reference's
// Solver::writeToFile_ (solution file in OUTPUT_FORMAT, slip-wall CSV when OUTPUT_SLIP_WALL).
// With geometry it writes the geometry alone (the operator dumps are 3-D only).
#include "fluxroe_return_fix.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

// SolverImplicit keeps its state private (and Solver protected); the harness reads it, so
// only in this translation unit those members are made accessible (layout is unchanged).
#define private public
#define protected public
#include "SolverImplicit.hpp"
#undef protected
#undef private
#include "SolverExplicit.hpp"

namespace {

std::string g_out;
// Dimension of the mesh and conserved-variable count.  Every output keeps the 3-D layout
// ([3] coordinates, [4] local faces, [5] variables); a 2-D mesh's missing entries are zero
// (face ids -1) and its variables (rho, rho u, rho v, rho E) go to slots 0, 1, 2, 4.
int g_nd = 3, g_nv = 5;
inline int slot5(int v) { return (g_nv == 5 || v < 3) ? v : 4; }

void write_bin(const std::string& name, const void* data, size_t bytes) {
  FILE* f = std::fopen((g_out + "/" + name).c_str(), "wb");
  if (!f) {
    std::fprintf(stderr, "cannot write %s\n", name.c_str());
    std::exit(2);
  }
  if (bytes) std::fwrite(data, 1, bytes, f);
  std::fclose(f);
}

void write_vec(const std::string& name, const std::vector<double>& v) {
  write_bin(name, v.data(), v.size() * sizeof(double));
}
void write_ivec(const std::string& name, const std::vector<long long>& v) {
  write_bin(name, v.data(), v.size() * sizeof(long long));
}

int boundary_code(BoundaryType t) {
  switch (t) {
    case BoundaryType::INTERNAL: return 0;
    case BoundaryType::SLIP_WALL: return 1;
    case BoundaryType::FREESTREAM: return 2;
  }
  return -1;
}

class HarnessExplicit : public SolverExplicit {
 public:
  void step(unsigned long it) { timeStep_(it, privateVariable_, g_out + "/ref_residual.csv"); }
  double** sub_residual() { return subResidual_; }
  Solution* solution() { return solution_; }
  Gradient* gradient() { return gradient_; }
  Limiter* limiter() { return limiter_; }
  TimeStepCalculator* dt() { return timeStepCalculator_; }
  void face_states(SolutionSnapshot* s, unsigned long f, double* l, double* r) {
    computeFaceConservedVariable_(s, gradient_, limiter_, f, l, r);
  }
};

void dump_geometry(Mesh* mesh) {
  const unsigned long nc = mesh->getNumElement(), nf = mesh->getNumFace();
  std::vector<double> vol(nc), cen(nc * 3), r(nc * 12), w(nc * 4);
  std::vector<long long> cface(nc * 4), cadj(nc * 4);
  for (unsigned long i = 0; i < nc; ++i) {
    Element* e = mesh->getElement(i);
    vol[i] = e->getVolume();
    for (int d = 0; d < g_nd; ++d) cen[i * 3 + d] = e->getCentroid()->getSingleCoord(d);
    for (int m = 0; m < 4; ++m) {
      if (m > g_nd) {  // 2-D: three faces per cell
        cface[i * 4 + m] = -1;
        cadj[i * 4 + m] = -1;
        continue;
      }
      cface[i * 4 + m] = (long long)e->getSingleFace(m)->getId();
      Element* a = e->getFaceAdjacentElement(m);
      cadj[i * 4 + m] = a ? (long long)a->getId() : -1;
      w[i * 4 + m] = e->getFaceInverseDistanceWeight(m);
      for (int d = 0; d < g_nd; ++d) r[i * 12 + m * 3 + d] = e->getVectorToFace(m)[d];
    }
  }
  std::vector<double> S(nf * 3), n(nf * 3), area(nf), fc(nf * 3);
  std::vector<long long> own(nf), nei(nf), typ(nf);
  for (unsigned long f = 0; f < nf; ++f) {
    Face* F = mesh->getFace(f);
    for (int d = 0; d < g_nd; ++d) {
      S[f * 3 + d] = F->getDimNormal()[d];
      n[f * 3 + d] = F->getNonDimNormal()[d];
      fc[f * 3 + d] = F->getCenter()->getSingleCoord(d);
    }
    area[f] = F->getArea();
    own[f] = (long long)F->getOwnerElement()->getId();
    nei[f] = F->getNeighborElement() ? (long long)F->getNeighborElement()->getId() : -1;
    typ[f] = boundary_code(F->getBoundaryType());
  }
  write_vec("geo_volume.bin", vol);
  write_vec("geo_centroid.bin", cen);
  write_vec("geo_vec_to_face.bin", r);
  write_vec("geo_weight.bin", w);
  write_ivec("geo_cell_face.bin", cface);
  write_ivec("geo_cell_adj.bin", cadj);
  write_vec("geo_face_S.bin", S);
  write_vec("geo_face_n.bin", n);
  write_vec("geo_face_area.bin", area);
  write_vec("geo_face_center.bin", fc);
  write_ivec("geo_face_owner.bin", own);
  write_ivec("geo_face_neigh.bin", nei);
  write_ivec("geo_face_type.bin", typ);
}

// MUSCL reconstruction looks the cell->face vector up through Element's face-id map
// (src/Element.cpp:185-187).  Record which local face each (cell, face) lookup resolves to,
// after the solver has run (the lookup inserts missing keys with local index 0).
void dump_muscl_face_slots(Mesh* mesh) {
  const unsigned long nc = mesh->getNumElement();
  std::vector<long long> slot(nc * 4, -1);
  for (unsigned long i = 0; i < nc; ++i) {
    Element* e = mesh->getElement(i);
    for (int m = 0; m <= g_nd; ++m) {
      const unsigned long fid = e->getSingleFace(m)->getId();
      const double* v = e->getVectorToFaceFromFaceId(fid);
      for (int k = 0; k <= g_nd; ++k)
        if (v == e->getVectorToFace(k)) slot[i * 4 + m] = k;
    }
  }
  write_ivec("geo_muscl_slot.bin", slot);
}

void norms_of(double** R, unsigned long nc, double* out10) {
  for (int k = 0; k < 10; ++k) out10[k] = 0.0;
  for (int v = 0; v < g_nv; ++v) {
    double s = 0.0, mx = 0.0;
    for (unsigned long i = 0; i < nc; ++i) {
      const double a = R[i][v];
      s += a * a;
      mx = std::fabs(a) > mx ? std::fabs(a) : mx;
    }
    out10[slot5(v)] = std::sqrt(s);
    out10[5 + slot5(v)] = mx;
  }
}

// state of a snapshot in the 3-D layout [nc][5]
std::vector<double> state_of(SolutionSnapshot* s, unsigned long nc) {
  std::vector<double> U(nc * 5, 0.0);
  for (unsigned long i = 0; i < nc; ++i)
    for (int v = 0; v < g_nv; ++v) U[i * 5 + slot5(v)] = s->getConservedVariable(i, (short)v);
  return U;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s case.besi outdir n_steps [explicit|implicit] [dump_ops]\n",
                 argv[0]);
    return 2;
  }
  const std::string besi = argv[1];
  g_out = argv[2];
  const unsigned long nsteps = std::strtoul(argv[3], nullptr, 10);
  bool dump_ops = false, write_out = false, dump_geo = false;
  for (int a = 5; a < argc; ++a) {
    dump_ops |= std::string(argv[a]) == "dump_ops";
    dump_geo |= std::string(argv[a]) == "geometry";
    write_out |= std::string(argv[a]) == "write";
  }

  Config* config = new Config();
  Mesh* mesh = new Mesh();
  Gas* gas = new GasPerfect();
  config->initialize(besi);
  mesh->initialize(config);
  config->initializePostMesh(mesh);
  gas->initialize(config);
  const unsigned long nc = mesh->getNumElement(), nf = mesh->getNumFace();
  g_nd = mesh->getNumDim();
  g_nv = config->getNumConservedVariable();
  if (g_nd != 3 && (dump_ops || (argc > 4 && std::string(argv[4]) == "kat"))) {
    std::fprintf(stderr, "operator dumps and known-answer records are 3-D only\n");
    return 2;
  }
  if (argc > 4 && std::string(argv[4]) == "kat") {
    // Known-answer mode: n records of (UL[5], UR[5], nhat[3]) from outdir/kat_in.bin through
    // the reference's flux and flux-Jacobian objects.  Output per record: Roe F[5], JL[25],
    // JR[25]; slip wall F[5], JL[25]; freestream F[5], JL[25].
    std::vector<double> in(nsteps * 13);
    FILE* f = std::fopen((g_out + "/kat_in.bin").c_str(), "rb");
    if (!f || std::fread(in.data(), 8, in.size(), f) != in.size()) {
      std::fprintf(stderr, "cannot read kat_in.bin\n");
      return 2;
    }
    std::fclose(f);
    FluxRoe roe;
    FluxFreestream fs;
    FluxSlipWall sw;
    roe.initialize(config, gas);
    fs.initialize(config, gas);
    sw.initialize(config, gas);
    FluxJacobianRoeThreeDim jroe;
    FluxJacobianFreestreamThreeDim jfs;
    FluxJacobianSlipWallThreeDim jsw;
    jroe.initialize(config);
    jfs.initialize(config);
    jsw.initialize(config);
    const int rec = 5 + 25 + 25 + 5 + 25 + 5 + 25;
    std::vector<double> out(nsteps * rec);
    double* pinf = config->getFreestreamPrimitiveVariables(0);
    for (unsigned long i = 0; i < nsteps; ++i) {
      const double* UL = &in[i * 13];
      const double* UR = UL + 5;
      const double* n = UL + 10;
      double* o = &out[i * rec];
      roe.computeFlux(UL, UR, n, o);
      jroe.computeJacobian(UL, UR, n, o + 5, o + 30);
      sw.computeFlux(UL, nullptr, n, o + 55);
      jsw.computeJacobian(UL, nullptr, n, o + 60, nullptr);
      fs.computeFlux(UL, pinf, n, o + 85);
      jfs.computeJacobian(UL, pinf, n, o + 90, nullptr);
    }
    write_vec("kat_out.bin", out);
    std::_Exit(0);
  }
  if (dump_ops || dump_geo) dump_geometry(mesh);

  if (config->getSolverType() == SolverType::EXPLICIT) {
    HarnessExplicit* solver = new HarnessExplicit();
    solver->initialize(config, gas, mesh);
    solver->setUniversalInitialCondition(config->getFreestreamPrimitiveVariables(0));
    std::vector<double> hist;
    for (unsigned long it = 0; it < nsteps; ++it) {
      if (dump_ops && it == 0) {
        SolutionSnapshot* s = solver->solution()->getCurrentSnapshot(0, 0);
        // perturb nothing: operators at the initial (uniform) state are trivial, so the
        // operator dump is taken after the first step instead (see below).
        (void)s;
      }
      solver->step(it);
      double nrm[10];
      norms_of(solver->sub_residual(), nc, nrm);
      hist.insert(hist.end(), nrm, nrm + 10);
      if (dump_ops && it + 1 == std::min<unsigned long>(nsteps, 3)) {
        // Operators evaluated on the state after it+1 steps (snapshot 0 of step it+1).
        SolutionSnapshot* s = solver->solution()->getCurrentSnapshot(it + 1, 0);
        std::vector<double> U(nc * 5);
        for (unsigned long i = 0; i < nc; ++i)
          for (int v = 0; v < 5; ++v) U[i * 5 + v] = s->getConservedVariable(i, (short)v);
        write_vec("op_state.bin", U);
        solver->dt()->computeAllTimeStep(s, config->getCourantNum());
        std::vector<double> dt(nc);
        for (unsigned long i = 0; i < nc; ++i) dt[i] = solver->dt()->getTimeStep(i);
        write_vec("op_dt.bin", dt);
        solver->gradient()->computeGradient(s);
        solver->limiter()->computeLimiterTerm(s, solver->gradient());
        std::vector<double> G(nc * 15), L(nc * 5);
        for (unsigned long i = 0; i < nc; ++i)
          for (int v = 0; v < 5; ++v) {
            L[i * 5 + v] = solver->limiter()->getLimiterValue(i, (short)v);
            for (int d = 0; d < 3; ++d)
              G[i * 15 + v * 3 + d] = solver->gradient()->getGradient(i, (short)v, (short)d);
          }
        write_vec("op_grad.bin", G);
        write_vec("op_limiter.bin", L);
        std::vector<double> UL(nf * 5), UR(nf * 5), F(nf * 5);
        FluxRoe roe;
        FluxFreestream fs;
        FluxSlipWall sw;
        roe.initialize(config, gas);
        fs.initialize(config, gas);
        sw.initialize(config, gas);
        for (unsigned long f = 0; f < nf; ++f) {
          solver->face_states(s, f, &UL[f * 5], &UR[f * 5]);
          Face* face = mesh->getFace(f);
          switch (face->getBoundaryType()) {
            case BoundaryType::INTERNAL:
              roe.computeFlux(&UL[f * 5], &UR[f * 5], face->getNonDimNormal(), &F[f * 5]);
              break;
            case BoundaryType::FREESTREAM:
              fs.computeFlux(&UL[f * 5], config->getFreestreamPrimitiveVariables(0),
                             face->getNonDimNormal(), &F[f * 5]);
              break;
            case BoundaryType::SLIP_WALL:
              sw.computeFlux(&UL[f * 5], nullptr, face->getNonDimNormal(), &F[f * 5]);
              break;
          }
        }
        write_vec("op_face_UL.bin", UL);
        write_vec("op_face_UR.bin", UR);
        write_vec("op_face_flux.bin", F);
      }
    }
    write_vec("residual_history.bin", hist);
    // the reference's own writers, called as its solve loop does after the last step
    // (src/SolverExplicit.cpp:427-433): solution_<n>.vtk|csv and slip_wall_<n>.csv
    if (write_out) solver->writeToFile_(nsteps - 1, config->getNumCurrentSolution() - 1);
    write_vec("final_state.bin", state_of(solver->solution()->getCurrentSnapshot(nsteps, 0), nc));
    if (dump_ops || dump_geo) dump_muscl_face_slots(mesh);
  } else {
    SolverImplicit* solver = new SolverImplicit();
    solver->initialize(config, gas, mesh);
    solver->setUniversalInitialCondition(config->getFreestreamPrimitiveVariables(0));
    std::vector<double> hist;  // per step: L2[5] of RHS, max[5] of RHS, iters, err, cfl
    for (unsigned long it = 0; it < nsteps; ++it) {
      const double cfl_used = solver->actualCourantNum_;
      solver->timeStep_(it, solver->faceLoopVariables_, g_out + "/ref_residual.csv");
      double l2[5] = {0, 0, 0, 0, 0}, mx[5] = {0, 0, 0, 0, 0};
      for (unsigned long i = 0; i < nc; ++i)
        for (int v = 0; v < g_nv; ++v) {
          const double x = solver->explicitFlux_[i * g_nv + v];
          l2[slot5(v)] += x * x;
        }
      for (int v = 0; v < g_nv; ++v) mx[slot5(v)] = solver->maxResidual_[v];
      for (int v = 0; v < 5; ++v) hist.push_back(std::sqrt(l2[v]));
      for (int v = 0; v < 5; ++v) hist.push_back(mx[v]);
      hist.push_back(cfl_used);
      hist.push_back(solver->actualCourantNum_);
      if (dump_ops && it == 0) {
        write_vec("op_rhs.bin", solver->explicitFlux_);
        write_vec("op_delta.bin", solver->deltaConservedVariable_);
        MatrixSparse* A = solver->coefficientMatrix_->getMatrixSparse();
        const ptrdiff_t nr = A->getNumRow();
        std::vector<long long> rp(A->getRowPtr(), A->getRowPtr() + nr + 1);
        std::vector<long long> cp(A->getColPtr(), A->getColPtr() + rp[nr]);
        std::vector<double> vp(A->getValPtr(), A->getValPtr() + rp[nr]);
        write_ivec("op_mat_rowptr.bin", rp);
        write_ivec("op_mat_col.bin", cp);
        write_vec("op_mat_val.bin", vp);
      }
    }
    write_vec("implicit_history.bin", hist);
    if (write_out) solver->writeToFile_(nsteps - 1, config->getNumCurrentSolution() - 1);
    write_vec("final_state.bin", state_of(solver->solution_->getCurrentSnapshot(nsteps, 0), nc));
    if (dump_ops || dump_geo) dump_muscl_face_slots(mesh);
  }
  std::fflush(stdout);
  // The reference's destructors loop with 16-bit counters over cells
  // (src/SolutionSnapshot.cpp:34-48) and fail beyond 32767 cells; skip them.
  std::_Exit(0);
}
