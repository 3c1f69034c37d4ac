// Solution output and the solve loop.
//
// The writers reproduce the reference's files text for text (joel-ho/BES
// src/SolutionSnapshot.cpp:145-309): the same layout, variable names and number formatting
// (a std::ofstream with its default flags, i.e. 6 significant digits), from the state in the
// reference's cell numbering.  Quantities written are the "dimensional" primitive variables of
// GasPerfect_<T>::convertDimensional (src/GasPerfect.tpp:294-326): rho, the Mach vector
// u/c(T), gamma*p and gamma*R*T, computed from the conserved state by
// GasPerfect_<T>::computeAllPrimitiveVariable (src/GasPerfect.tpp:34-111).
//
// bes_solve is Solver::solve (src/SolverExplicit.cpp:395-438, src/SolverImplicit.cpp:552-600):
// residual.csv is truncated, every step appends "<step>," and the residual line that
// timeStep_ logs (explicit: max |R| per variable of the last stage; implicit: max |RHS| per
// variable, linear iterations and linear error), and the solution (plus the slip-wall file when
// enabled) is written after step k when k % SAVE_INTERVAL == 0 and after the last step.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "context.hpp"

namespace {

void set_err(char* err, size_t cap, const std::string& msg) {
  if (err && cap) std::snprintf(err, cap, "%s", msg.c_str());
}

// dimensional primitive variables [rho, Mx, My, Mz, gamma*p, gamma*R*T] of one cell
void dimensional_primitive(const double* U, double gamma, double R, double* d) {
  const double cv = R / (gamma - 1.0);
  const double rho = U[0];
  double u[3];
  for (int k = 0; k < 3; ++k) u[k] = U[1 + k] / U[0];
  double q = 0.0;
  for (int k = 0; k < 3; ++k) q += U[1 + k] * U[1 + k];
  const double p = (gamma - 1.0) * (U[4] - q / (2.0 * U[0]));
  const double T = (1.0 / (cv * U[0])) * (U[4] - q / (2.0 * U[0]));
  d[0] = rho;
  d[4] = gamma * p;
  d[5] = gamma * R * T;
  const double c = std::sqrt(gamma * R * T);
  for (int k = 0; k < 3; ++k) d[1 + k] = u[k] / c;
}

struct OutMesh {
  const bes::RefMesh* ref;
  const double* nodes;
  int64_t n_nodes;
  const int64_t* tets;
};

int write_file(const OutMesh& m, const double* U, double gamma, double R, const char* path,
               int kind, std::string& err) {
  const bes::RefMesh& M = *m.ref;
  const int64_t nc = M.nc;
  std::vector<double> D((size_t)nc * 6);
  for (int64_t i = 0; i < nc; ++i) dimensional_primitive(U + i * 5, gamma, R, &D[i * 6]);
  std::ofstream out(path);
  if (!out) {
    err = std::string("cannot open ") + path + " for writing";
    return BES_ERR_INVALID;
  }
  // primitive columns: rho, the nd velocity (Mach) components, p, T
  const int nd = M.dim;
  const int nvc = nd + 1;  // vertices per cell
  int pcols[6], np = 0;
  pcols[np++] = 0;
  for (int k = 0; k < nd; ++k) pcols[np++] = 1 + k;
  pcols[np++] = 4;
  pcols[np++] = 5;
  if (kind == BES_OUTPUT_CSV) {  // SolutionSnapshot::writePrimitiveToCsv
    for (int64_t i = 0; i < nc; ++i) {
      for (int k = 0; k < nd; ++k) out << M.centroid[i * 3 + k] << ",";
      for (int v = 0; v < np; ++v) out << D[i * 6 + pcols[v]] << ",";
      out << "\n";
    }
  } else if (kind == BES_OUTPUT_VTK) {  // SolutionSnapshot::writePrimitiveToVtk
    out << "# vtk DataFile Version 2.0\n" << path << "\nASCII\nDATASET UNSTRUCTURED_GRID\n";
    out << "POINTS " << m.n_nodes << " float\n";
    for (int64_t v = 0; v < m.n_nodes; ++v) {
      for (int k = 0; k < nd; ++k) out << m.nodes[v * 3 + k] << " ";
      if (nd == 2) out << 0.0 << " ";
      out << "\n";
    }
    out << "CELLS " << nc << " " << nc * (nvc + 1) << "\n";
    for (int64_t i = 0; i < nc; ++i) {
      out << nvc << " ";
      for (int k = 0; k < nvc; ++k) out << m.tets[i * nvc + k] << " ";
      out << "\n";
    }
    out << "CELL_TYPES " << nc << "\n";
    // VTK_TETRA 10 (ElementGmshFour), VTK_TRIANGLE 5 (ElementGmshTwo)
    for (int64_t i = 0; i < nc; ++i) out << (nd == 3 ? 10 : 5) << "\n";
    out << "CELL_DATA " << nc << "\n";
    const char* names[3] = {"rho_nondim", "P_nondim", "T_nondim"};
    const int cols[3] = {0, 4, 5};
    for (int s = 0; s < 3; ++s) {
      out << "SCALARS " << names[s] << " double\nLOOKUP_TABLE default\n";
      for (int64_t i = 0; i < nc; ++i) out << D[i * 6 + cols[s]] << "\n";
    }
    out << "VECTORS M double\n";
    for (int64_t i = 0; i < nc; ++i) {
      for (int k = 0; k < nd; ++k) out << D[i * 6 + 1 + k] << " ";
      if (nd == 2) out << 0.0 << " ";
      out << "\n";
    }
  } else if (kind == BES_OUTPUT_SLIP_WALL_CSV) {  // SolutionSnapshot::writeSlipWallToCsv
    for (int64_t f = 0; f < M.nf; ++f) {
      if (M.kind[f] != 1) continue;
      const int64_t o = M.owner[f];
      for (int k = 0; k < nd; ++k) out << M.center[f * 3 + k] << ",";
      for (int k = 0; k < nd; ++k) out << M.S[f * 3 + k] << ",";
      for (int v = 0; v < np; ++v) out << D[o * 6 + pcols[v]] << ",";
      out << "\n";
    }
  } else {
    err = "unknown output kind";
    return BES_ERR_INVALID;
  }
  out.flush();
  if (!out) {
    err = std::string("write error on ") + path;
    return BES_ERR_INVALID;
  }
  return BES_OK;
}

}  // namespace

extern "C" {

void bes_output_default(bes_output* o) {
  std::memset(o, 0, sizeof(*o));
  std::snprintf(o->folder, sizeof(o->folder), ".");
  o->format = BES_OUTPUT_VTK;
  o->slip_wall = 0;
  o->save_interval = 0;
  o->verbose = 0;
}

int bes_write_host(const bes_mesh_arrays* mesh, const bes_options* opt, const double* U,
                   const char* path, int32_t kind, char* err, size_t err_cap) {
  if (!mesh || !opt || !U || !path) return BES_ERR_INVALID;
  bes::RefMesh M;
  std::string e;
  if (!bes::build_ref_mesh(mesh->nodes, mesh->n_nodes, mesh->btris, mesh->btags, mesh->n_btris,
                           mesh->tets, mesh->n_tets, bes_mesh_dim(mesh),
                           opt->muscl_face_vector != 0, M, e)) {
    set_err(err, err_cap, e);
    return BES_ERR_MESH;
  }
  OutMesh m{&M, mesh->nodes, mesh->n_nodes, mesh->tets};
  const int rc = write_file(m, U, opt->specific_heat_ratio, opt->gas_constant, path, kind, e);
  if (rc) set_err(err, err_cap, e);
  return rc;
}

int bes_write(bes_ctx* ctx, const char* path, int32_t kind) {
  if (!ctx || !path) return BES_ERR_INVALID;
  // batched contexts: the first condition
  std::vector<double> U((size_t)ctx->soa.nc * 5 * ctx->nb);
  int rc = bes_get_state(ctx, U.data());
  if (rc) return rc;
  OutMesh m{&ctx->ref, ctx->nodes.data(), (int64_t)(ctx->nodes.size() / 3), ctx->tets.data()};
  std::string e;
  rc = write_file(m, U.data(), ctx->opt.specific_heat_ratio, ctx->opt.gas_constant, path, kind, e);
  if (rc) ctx->last_error = e;
  return rc;
}

int bes_solve(bes_ctx* ctx, const bes_output* out) {
  if (!ctx || !out) return BES_ERR_INVALID;
  if (ctx->nb != 1) {
    ctx->last_error = "bes_solve runs single-condition contexts (bes_sweep_run runs batches)";
    return BES_ERR_UNSUPPORTED;
  }
  const bes_options& o = ctx->opt;
  const int64_t nsteps = o.number_of_time_step;
  const bool implicit = o.solver_type == 1;
  const std::string folder = out->folder;
  const std::string res_path = folder + "/residual.csv";
  { std::ofstream trunc(res_path); if (!trunc) { ctx->last_error = "cannot open " + res_path; return BES_ERR_INVALID; } }
  // conserved variables of the mesh dimension: a 2-D mesh has no rho w
  const int nvar = ctx->ref.dim + 2;
  const int vars[5] = {0, 1, 2, nvar == 4 ? 4 : 3, 4};
  if (out->verbose) {
    std::cout << "Running solver on the GPU..." << std::endl << std::endl;
    std::cout << "  | Time step | ";
    for (int v = 0; v < nvar; ++v) std::cout << "Conserved variable " << (v + 1) << " | ";
    std::cout << std::endl;
  }
  const int ncol = implicit ? 19 : 10;
  std::vector<double> hist;
  int64_t it = 0;
  while (it < nsteps) {
    // run up to (and including) the next step after which a file is written
    int64_t last = nsteps - 1;
    if (out->save_interval > 0) {
      const int64_t k = out->save_interval;
      const int64_t next = (it % k == 0) ? it : (it / k + 1) * k;
      last = std::min(last, next);
    }
    const int64_t n = last - it + 1;
    hist.assign((size_t)n * ncol, 0.0);
    const int rc = implicit ? bes_implicit_steps(ctx, n, hist.data())
                            : bes_explicit_iterations(ctx, n, hist.data());
    if (rc) return rc;
    std::ofstream res(res_path, std::ios::app);
    for (int64_t q = 0; q < n; ++q) {
      const double* h = &hist[(size_t)q * ncol];
      std::ostringstream line, con;
      line << (it + q + 1) << ",";
      line << std::scientific;
      con << std::scientific << "  | " << (it + q + 1) << " | ";
      for (int k = 0; k < nvar; ++k) {
        line << h[5 + vars[k]] << ",";
        con << h[5 + vars[k]] << " | ";
      }
      if (implicit) {
        line << (int64_t)h[12] << "," << h[13] << ",";
        con << (int64_t)h[12] << " | " << h[13] << " | ";
      }
      line << "\n";
      res << line.str();
      if (out->verbose) std::cout << con.str() << std::endl;
    }
    res.close();
    const std::string step = std::to_string(last + 1);
    const bool vtk = out->format == BES_OUTPUT_VTK;
    int wrc = bes_write(ctx, (folder + "/solution_" + step + (vtk ? ".vtk" : ".csv")).c_str(),
                        vtk ? BES_OUTPUT_VTK : BES_OUTPUT_CSV);
    if (wrc) return wrc;
    if (out->slip_wall) {
      wrc = bes_write(ctx, (folder + "/slip_wall_" + step + ".csv").c_str(),
                      BES_OUTPUT_SLIP_WALL_CSV);
      if (wrc) return wrc;
    }
    it = last + 1;
  }
  if (out->verbose) std::cout << std::endl << "Solver run completed." << std::endl;
  return BES_OK;
}

}  // extern "C"
