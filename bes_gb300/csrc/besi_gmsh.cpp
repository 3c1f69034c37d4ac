// .besi option files and Gmsh 2.2 ASCII meshes.
//
// bes_options_from_besi follows Config::readConfigFile_ (src/Config.cpp:116-422 of
// joel-ho/BES): a line is cut at "//", split at "=", and every blank, tab and carriage return is
// removed from key and value (ReadFile::trimWhiteSpace removes them everywhere, not only at the
// ends); values are comma separated; an unknown non-empty key is an error.  Keys added by this
// library are listed in ADDITIVE_KEYS below.
//
// bes_mesh_read_gmsh follows Mesh::readGmsh (src/Mesh.cpp:95-558): node ids are ignored and
// nodes are numbered in file order; element node references are 1-based; triangles (type 2)
// are boundary faces whose first tag names a physical group SLIP_WALL or FREESTREAM;
// tetrahedra (type 4) are cells; other element types are skipped.  When the largest physical
// name dimension is 2 (2-D), lines (type 1) are the boundary faces and triangles the cells.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/bes_gb300.h"
#include "mesh_host.hpp"

namespace {

std::string strip_all(const std::string& s) {
  std::string o;
  o.reserve(s.size());
  for (char ch : s)
    if (ch != ' ' && ch != '\t' && ch != '\r' && ch != '\0') o.push_back(ch);
  return o;
}

std::vector<std::string> split(const std::string& s, const std::string& delim) {
  std::vector<std::string> out;
  size_t start = 0, end;
  while ((end = s.find(delim, start)) != std::string::npos) {
    out.push_back(strip_all(s.substr(start, end - start)));
    start = end + delim.size();
  }
  out.push_back(strip_all(s.substr(start)));
  return out;
}

bool to_num(const std::string& s, double& x) {
  if (s.empty()) return false;
  char* e = nullptr;
  errno = 0;
  x = std::strtod(s.c_str(), &e);
  return e && *e == '\0' && errno == 0;
}

void set_err(char* err, size_t cap, const std::string& msg) {
  if (err && cap) std::snprintf(err, cap, "%s", msg.c_str());
}

}  // namespace

extern "C" int bes_options_from_besi(const char* path, bes_options* o, char* mesh_path,
                                     size_t mesh_path_cap, char* err, size_t err_cap) {
  if (!path || !o) return BES_ERR_INVALID;
  bes_options_default(o);
  std::ifstream in(path);
  if (!in) {
    set_err(err, err_cap, std::string("cannot open ") + path);
    return BES_ERR_CONFIG;
  }
  std::string line, mesh_file;
  int lineno = 0;
  auto bad = [&](const std::string& m) {
    set_err(err, err_cap, "line " + std::to_string(lineno) + ": " + m);
    return BES_ERR_CONFIG;
  };
  while (std::getline(in, line)) {
    ++lineno;
    const std::string body = line.substr(0, line.find("//"));
    std::vector<std::string> kv = split(body, "=");
    const std::string key = kv[0];
    if (key.empty()) continue;
    const std::string val = kv.size() > 1 ? kv[1] : "";
    std::vector<std::string> args = split(val, ",");
    std::vector<double> nums;
    for (auto& a : args) {
      double x;
      nums.push_back(to_num(a, x) ? x : std::nan(""));
    }
    auto word = [&](std::initializer_list<const char*> allowed) -> int {
      int i = 0;
      for (const char* w : allowed) {
        if (args[0] == w) return i;
        ++i;
      }
      return -1;
    };
    auto num = [&](size_t i, double& x) {
      if (i >= nums.size() || nums[i] != nums[i]) return false;
      x = nums[i];
      return true;
    };
    double x = 0;
    if (key == "MESH_FORMAT") {
      if (word({"GMSH"}) < 0) return bad("Mesh format not supported");
    } else if (key == "MESH_FILE") {
      mesh_file = args[0];
    } else if (key == "OUTPUT_FORMAT") {
      if (word({"VTK", "CSV"}) < 0) return bad("Output format not supported");
    } else if (key == "OUTPUT_SLIP_WALL") {
      if (word({"YES", "NO"}) < 0) return bad("Output slip wall format not supported");
    } else if (key == "OUTPUT_FOLDER") {
    } else if (key == "EQUATION") {
      if (word({"EULER_NON_DIMENSIONAL"}) < 0) return bad("Equation not supported");
    } else if (key == "SOLVER_TYPE") {
      const int w = word({"EXPLICIT", "IMPLICIT"});
      if (w < 0) return bad("Solver type not supported");
      o->solver_type = w;
    } else if (key == "EXPLICIT_SCHEME") {
      if (word({"MULTI_STEP"}) < 0) return bad("Explicit scheme not supported");
    } else if (key == "MULTI_TIME_STEP_OPTIONS") {
      if (!num(0, x) || x < 1 || x > 8) return bad("MULTI_TIME_STEP_OPTIONS needs 1..8 stages");
      o->n_stage = (int32_t)x;
      for (int k = 0; k < o->n_stage; ++k)
        if (!num(1 + k, o->stage_coeff[k])) return bad("missing multi-step coefficient");
    } else if (key == "COURANT_NUM") {
      if (!num(0, o->courant_num)) return bad("bad COURANT_NUM");
    } else if (key == "ADAPTIVE_COURANT_NUM_MAX") {
      if (!num(0, o->adaptive_courant_num_max)) return bad("bad ADAPTIVE_COURANT_NUM_MAX");
    } else if (key == "ADAPTIVE_COURANT_NUM_EXPONENT") {
      if (!num(0, o->adaptive_courant_num_exponent[0]) || !num(1, o->adaptive_courant_num_exponent[1]))
        return bad("ADAPTIVE_COURANT_NUM_EXPONENT needs two numbers");
    } else if (key == "LOCAL_TIME_STEP") {
      const int w = word({"YES", "NO"});
      if (w < 0) return bad("Local time step option not supported");
      o->local_time_step = (w == 0);
    } else if (key == "NUMBER_OF_TIME_STEP") {
      if (!num(0, x)) return bad("bad NUMBER_OF_TIME_STEP");
      o->number_of_time_step = (int32_t)x;
    } else if (key == "SAVE_INTERVAL") {
      if (!num(0, x)) return bad("bad SAVE_INTERVAL");
    } else if (key == "FREESTREAM_RAMP") {
      if (!num(0, x) || x < 0) return bad("bad FREESTREAM_RAMP");
      o->freestream_ramp = (int32_t)x;
    } else if (key == "FREESTREAM_RAMP_START_FRAC") {
      if (!num(0, o->freestream_ramp_start_frac)) return bad("bad FREESTREAM_RAMP_START_FRAC");
    } else if (key == "GRADIENT_SCHEME") {
      if (word({"GREEN_GAUSS"}) < 0) return bad("Gradient scheme not supported");
    } else if (key == "LIMITER_SCHEME") {
      if (word({"VENKATAKRISHNAN"}) < 0) return bad("Limiter not supported");
    } else if (key == "VENKATAKRISHNAN_FACTOR") {
      if (!num(0, o->venkatakrishnan_factor)) return bad("bad VENKATAKRISHNAN_FACTOR");
    } else if (key == "HARTEN_CORRECTION_LIMIT") {
      if (!num(0, o->harten_correction_limit)) return bad("bad HARTEN_CORRECTION_LIMIT");
    } else if (key == "FLUX_SCHEME") {
      if (word({"ROE"}) < 0) return bad("Flux discretization scheme not supported");
    } else if (key == "GAS_CONSTANT") {
      if (!num(0, o->gas_constant)) return bad("bad GAS_CONSTANT");
    } else if (key == "SPECIFIC_HEAT_RATIO") {
      if (!num(0, o->specific_heat_ratio)) return bad("bad SPECIFIC_HEAT_RATIO");
    } else if (key == "FREESTREAM_MACH") {
      for (int d = 0; d < 3; ++d)
        if (!num(d, o->freestream_mach[d])) return bad("FREESTREAM_MACH needs three numbers");
    } else if (key == "LINEAR_SOLVER") {
      // FGMRES/GMRES/LGMRES/BICGSTAB (the reference's AMGCL solvers) all map to GMRES(m);
      // BLOCK_JACOBI_GMRES / BLOCK_ILU0_GMRES (colour order) / BLOCK_ILU0_RCM_GMRES (reverse
      // Cuthill-McKee order, level scheduled) select the preconditioner explicitly.
      const int w = word({"FGMRES", "GMRES", "LGMRES", "BICGSTAB", "BLOCK_JACOBI_GMRES",
                          "BLOCK_ILU0_GMRES", "BLOCK_ILU0_RCM_GMRES"});
      if (w < 0) return bad("Linear solver option not supported");
      if (w == 4) o->linear_solver = 0;
      if (w == 5) o->linear_solver = 1;
      if (w == 6) o->linear_solver = 2;
    } else if (key == "AMG_PRECOND_COARSENER") {
      if (word({"AGGREGATION", "SMOOTHED_AGGREGATION", "SMOOTHED_AGGREGATION_EMIN",
                "RUGE_STUBEN"}) < 0)
        return bad("AMG preconditioner coarsening option not supported");
    } else if (key == "AMG_PRECOND_SMOOTHER") {
      // the smoother becomes the single-level preconditioner: ILU0 -> block ILU(0), others ->
      // block Jacobi
      const int w = word({"DAMPED_JACOBI", "ILU0", "SPAI0", "GAUSS_SEIDEL"});
      if (w < 0) return bad("AMG preconditioner smoothening option not supported");
      o->linear_solver = (w == 1) ? 1 : 0;
    } else if (key == "LINEAR_SOLVER_MAX_ITER") {
      if (!num(0, x)) return bad("bad LINEAR_SOLVER_MAX_ITER");
      o->linear_solver_max_iter = (int32_t)x;
    } else if (key == "LINEAR_SOLVER_ABS_TOL") {
      if (!num(0, o->linear_solver_tol)) return bad("bad LINEAR_SOLVER_ABS_TOL");
    } else if (key == "MUSCL_FACE_VECTOR") {  // additive
      const int w = word({"REFERENCE", "EXACT"});
      if (w < 0) return bad("MUSCL_FACE_VECTOR must be REFERENCE or EXACT");
      o->muscl_face_vector = w;
    } else if (key == "GMRES_RESTART") {  // additive
      // the Gram-Schmidt kernels take the basis size as a compile-time constant, up to 32
      if (!num(0, x) || x < 1 || x > 32) return bad("GMRES_RESTART must be 1..32");
      o->gmres_restart = (int32_t)x;
    } else if (key == "PRECISION") {  // additive
      const int w = word({"FP64", "MIXED", "MIXED_PACKED"});
      if (w < 0) return bad("PRECISION must be FP64, MIXED or MIXED_PACKED");
      o->precision = w;
    } else if (key == "CFL_RAMP") {  // additive: steps, start, end
      double a, b;
      if (!num(0, x) || !num(1, a) || !num(2, b) || x < 0 || a <= 0 || b <= 0)
        return bad("CFL_RAMP needs steps, start CFL, end CFL");
      o->cfl_ramp_steps = (int32_t)x;
      o->cfl_ramp_start = a;
      o->cfl_ramp_end = b;
    } else if (key == "SWEEP_KERNEL") {  // additive
      const int w = word({"AUTO", "PER_COLOUR", "PERSISTENT", "PER_COLOUR_LOADS_FIRST"});
      if (w < 0)
        return bad("SWEEP_KERNEL must be AUTO, PER_COLOUR, PERSISTENT or PER_COLOUR_LOADS_FIRST");
      o->sweep_kernel = w;
    } else if (key == "JACOBIAN_REPEAT") {  // additive: without it, the reference's count
      if (!num(0, x) || x < 1) return bad("JACOBIAN_REPEAT must be >= 1");
      o->jacobian_repeat = (int32_t)x;
    } else {
      return bad("Option \"" + key + "\" not supported");
    }
  }
  if (mesh_path && mesh_path_cap) std::snprintf(mesh_path, mesh_path_cap, "%s", mesh_file.c_str());
  return BES_OK;
}

extern "C" int bes_mesh_read_gmsh(const char* path, bes_mesh_arrays* out, char* err,
                                  size_t err_cap) {
  if (!path || !out) return BES_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    set_err(err, err_cap, std::string("cannot open ") + path);
    return BES_ERR_MESH;
  }
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<char> buf((size_t)size + 1);
  if (size > 0 && std::fread(buf.data(), 1, (size_t)size, f) != (size_t)size) {
    std::fclose(f);
    set_err(err, err_cap, "read error");
    return BES_ERR_MESH;
  }
  std::fclose(f);
  buf[size] = '\0';
  char* p = buf.data();
  char* end = p + size;
  auto next_line = [&](std::string& s) -> bool {
    if (p >= end) return false;
    char* e = (char*)std::memchr(p, '\n', (size_t)(end - p));
    if (!e) e = end;
    s.assign(p, e);
    if (!s.empty() && s.back() == '\r') s.pop_back();
    p = e + 1;
    return true;
  };
  std::map<int, int> tag_kind;  // physical tag -> 1 slip, 2 freestream, 0 other
  std::vector<double> nodes;
  std::vector<int64_t> btris, tets;
  std::vector<int32_t> btags;
  std::string line;
  bool tet_seen = false;
  int nd = 0;  // largest physical-name dimension (Mesh::readGmsh's nDim_)
  while (next_line(line)) {
    if (line == "$PhysicalNames") {
      if (!next_line(line)) break;
      const long n = std::strtol(line.c_str(), nullptr, 10);
      for (long i = 0; i < n && next_line(line); ++i) {
        int dim = 0, tag = 0;
        char name[256] = {0};
        if (std::sscanf(line.c_str(), "%d %d \"%255[^\"]\"", &dim, &tag, name) >= 2) {
          nd = dim > nd ? dim : nd;
          const std::string nm(name);
          tag_kind[tag] = nm == "SLIP_WALL" ? 1 : (nm == "FREESTREAM" ? 2 : 0);
        }
      }
    } else if (line == "$Nodes") {
      if (!next_line(line)) break;
      const long n = std::strtol(line.c_str(), nullptr, 10);
      nodes.resize((size_t)n * 3);
      for (long i = 0; i < n; ++i) {
        char* q = p;
        std::strtol(q, &q, 10);  // node id (ignored, as in the reference)
        for (int d = 0; d < 3; ++d) nodes[i * 3 + d] = std::strtod(q, &q);
        char* e = (char*)std::memchr(p, '\n', (size_t)(end - p));
        p = e ? e + 1 : end;
      }
    } else if (line == "$Elements") {
      if (!next_line(line)) break;
      const long n = std::strtol(line.c_str(), nullptr, 10);
      for (long i = 0; i < n; ++i) {
        char* q = p;
        std::strtol(q, &q, 10);
        const long type = std::strtol(q, &q, 10);
        const long ntags = std::strtol(q, &q, 10);
        long tag0 = 0;
        for (long t = 0; t < ntags; ++t) {
          const long v = std::strtol(q, &q, 10);
          if (t == 0) tag0 = v;
        }
        const bool two_d = nd == 2;
        if (two_d && type == 1) {
          if (tet_seen) {
            set_err(err, err_cap,
                    "boundary line listed after a triangle (the reference's reader needs "
                    "boundary lines first)");
            return BES_ERR_MESH;
          }
          for (int k = 0; k < 2; ++k) btris.push_back(std::strtoll(q, &q, 10) - 1);
          auto it = tag_kind.find((int)tag0);
          const int kind = it == tag_kind.end() ? 0 : it->second;
          if (kind == 0) {
            set_err(err, err_cap, "Unknown boundary type entered (physical tag " +
                                      std::to_string(tag0) + ")");
            return BES_ERR_MESH;
          }
          btags.push_back(kind);
        } else if (two_d && type == 2) {
          tet_seen = true;
          for (int k = 0; k < 3; ++k) tets.push_back(std::strtoll(q, &q, 10) - 1);
        } else if (two_d && type == 4) {
          set_err(err, err_cap, "tetrahedron in a 2D problem");
          return BES_ERR_MESH;
        } else if (type == 2) {
          if (tet_seen) {
            set_err(err, err_cap,
                    "boundary triangle listed after a tetrahedron (the reference's reader needs "
                    "boundary triangles first)");
            return BES_ERR_MESH;
          }
          for (int k = 0; k < 3; ++k) btris.push_back(std::strtoll(q, &q, 10) - 1);
          auto it = tag_kind.find((int)tag0);
          const int kind = it == tag_kind.end() ? 0 : it->second;
          if (kind == 0) {
            set_err(err, err_cap, "Unknown boundary type entered (physical tag " +
                                      std::to_string(tag0) + ")");
            return BES_ERR_MESH;
          }
          btags.push_back(kind);
        } else if (type == 4) {
          tet_seen = true;
          for (int k = 0; k < 4; ++k) tets.push_back(std::strtoll(q, &q, 10) - 1);
        } else if (type == 1) {
          set_err(err, err_cap, "1D boundary encountered in 3D problem");
          return BES_ERR_MESH;
        }
        char* e = (char*)std::memchr(p, '\n', (size_t)(end - p));
        p = e ? e + 1 : end;
      }
    }
  }
  if (nodes.empty() || tets.empty()) {
    set_err(err, err_cap, "mesh has no nodes or no cells");
    return BES_ERR_MESH;
  }
  const int nvc = nd == 2 ? 3 : 4;
  double* X = (double*)std::malloc(nodes.size() * sizeof(double));
  int64_t* T = (int64_t*)std::malloc(tets.size() * sizeof(int64_t));
  int64_t* B = (int64_t*)std::malloc((btris.size() + 1) * sizeof(int64_t));
  int32_t* BT = (int32_t*)std::malloc((btags.size() + 1) * sizeof(int32_t));
  std::memcpy(X, nodes.data(), nodes.size() * sizeof(double));
  std::memcpy(T, tets.data(), tets.size() * sizeof(int64_t));
  if (!btris.empty()) std::memcpy(B, btris.data(), btris.size() * sizeof(int64_t));
  if (!btags.empty()) std::memcpy(BT, btags.data(), btags.size() * sizeof(int32_t));
  out->n_nodes = (int64_t)nodes.size() / 3;
  out->nodes = X;
  out->n_tets = (int64_t)tets.size() / nvc;
  out->tets = T;
  out->dim = nd == 2 ? 2 : 3;
  out->n_btris = (int64_t)btags.size();
  out->btris = B;
  out->btags = BT;
  return BES_OK;
}

extern "C" void bes_mesh_free(bes_mesh_arrays* m) {
  if (!m) return;
  std::free((void*)m->nodes);
  std::free((void*)m->tets);
  std::free((void*)m->btris);
  std::free((void*)m->btags);
  std::memset(m, 0, sizeof(*m));
}

extern "C" void bes_abi_sizes(int64_t* out) {
  out[0] = (int64_t)sizeof(bes_options);
  out[1] = (int64_t)sizeof(bes_mesh_arrays);
  out[2] = (int64_t)sizeof(bes_output);
}

extern "C" int bes_output_from_besi(const char* path, bes_output* out, char* err,
                                    size_t err_cap) {
  if (!path || !out) return BES_ERR_INVALID;
  bes_output_default(out);
  std::ifstream in(path);
  if (!in) {
    set_err(err, err_cap, std::string("cannot open ") + path);
    return BES_ERR_CONFIG;
  }
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    std::vector<std::string> kv = split(line.substr(0, line.find("//")), "=");
    const std::string& key = kv[0];
    if (key.empty()) continue;
    const std::string arg = split(kv.size() > 1 ? kv[1] : "", ",")[0];
    auto bad = [&](const std::string& m) {
      set_err(err, err_cap, "line " + std::to_string(lineno) + ": " + m);
      return BES_ERR_CONFIG;
    };
    if (key == "OUTPUT_FOLDER") {
      std::snprintf(out->folder, sizeof(out->folder), "%s", arg.c_str());
    } else if (key == "OUTPUT_FORMAT") {
      if (arg == "VTK") out->format = BES_OUTPUT_VTK;
      else if (arg == "CSV") out->format = BES_OUTPUT_CSV;
      else return bad("Output format not supported");
    } else if (key == "OUTPUT_SLIP_WALL") {
      if (arg == "YES") out->slip_wall = 1;
      else if (arg == "NO") out->slip_wall = 0;
      else return bad("Output slip wall format not supported");
    } else if (key == "SAVE_INTERVAL") {
      double x;
      if (!to_num(arg, x) || x < 0) return bad("bad SAVE_INTERVAL");
      out->save_interval = (int64_t)x;
    }
  }
  return BES_OK;
}

extern "C" int bes_host_geometry(const bes_mesh_arrays* mesh, int32_t muscl_face_vector,
                                 int64_t* n_cells, int64_t* n_faces, double* volume,
                                 double* centroid, double* face_S, double* face_area,
                                 int64_t* face_owner, int64_t* face_neigh, int64_t* face_kind,
                                 int64_t* muscl_slot, int64_t* cell_new2ref,
                                 int64_t* face_new2ref, char* err, size_t err_cap) {
  if (!mesh) return BES_ERR_INVALID;
  bes::RefMesh M;
  std::string e;
  if (!bes::build_ref_mesh(mesh->nodes, mesh->n_nodes, mesh->btris, mesh->btags, mesh->n_btris,
                           mesh->tets, mesh->n_tets, bes_mesh_dim(mesh), muscl_face_vector != 0,
                           M, e)) {
    set_err(err, err_cap, e);
    return BES_ERR_MESH;
  }
  if (n_cells) *n_cells = M.nc;
  if (n_faces) *n_faces = M.nf;
  if (volume) std::memcpy(volume, M.vol.data(), M.nc * sizeof(double));
  if (centroid) std::memcpy(centroid, M.centroid.data(), M.nc * 3 * sizeof(double));
  if (face_S) std::memcpy(face_S, M.S.data(), M.nf * 3 * sizeof(double));
  if (face_area) std::memcpy(face_area, M.area.data(), M.nf * sizeof(double));
  if (face_owner) std::memcpy(face_owner, M.owner.data(), M.nf * sizeof(int64_t));
  if (face_neigh) std::memcpy(face_neigh, M.neigh.data(), M.nf * sizeof(int64_t));
  if (face_kind)
    for (int64_t f = 0; f < M.nf; ++f) face_kind[f] = M.kind[f];
  if (muscl_slot)
    for (int64_t q = 0; q < M.nc * 4; ++q) muscl_slot[q] = M.muscl_slot[q];
  if (cell_new2ref || face_new2ref) {
    bes::SoaMesh S;
    bes::build_soa(M, 5.0, muscl_face_vector != 0, true, S);
    if (cell_new2ref) std::memcpy(cell_new2ref, S.cell_new2ref.data(), M.nc * sizeof(int64_t));
    if (face_new2ref) std::memcpy(face_new2ref, S.face_new2ref.data(), M.nf * sizeof(int64_t));
  }
  return BES_OK;
}

namespace {
// FNV-1a over the bytes of an array
template <class T>
uint64_t digest_of(const std::vector<T>& v) {
  uint64_t h = 1469598103934665603ull;
  const unsigned char* p = reinterpret_cast<const unsigned char*>(v.data());
  for (size_t i = 0; i < v.size() * sizeof(T); ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h ^ (uint64_t)v.size();
}
}  // namespace

extern "C" int bes_host_layout_digest(const bes_mesh_arrays* mesh, int32_t muscl_face_vector,
                                      int32_t rcm_ilu_order, uint64_t* digests, int32_t cap,
                                      int32_t* n, char* err, size_t err_cap) {
  if (!mesh || !n) return BES_ERR_INVALID;
  bes::RefMesh M;
  std::string e;
  if (!bes::build_ref_mesh(mesh->nodes, mesh->n_nodes, mesh->btris, mesh->btags, mesh->n_btris,
                           mesh->tets, mesh->n_tets, bes_mesh_dim(mesh), muscl_face_vector != 0,
                           M, e)) {
    set_err(err, err_cap, e);
    return BES_ERR_MESH;
  }
  bes::SoaMesh S;
  bes::build_soa(M, 5.0, muscl_face_vector != 0, true, S);
  if (rcm_ilu_order) bes::build_ilu_schedule(S, true);
  const uint64_t d[] = {
      digest_of(S.cell_new2ref), digest_of(S.cell_ref2new), digest_of(S.face_new2ref),
      digest_of(S.face_ref2new), digest_of(S.vol), digest_of(S.inv_vol), digest_of(S.eps2),
      digest_of(S.plen), digest_of(S.adj), digest_of(S.cface), digest_of(S.gface),
      digest_of(S.Sc), digest_of(S.w), digest_of(S.r), digest_of(S.cflags),
      digest_of(S.extra_cell), digest_of(S.extra_m), digest_of(S.fown), digest_of(S.fnb),
      digest_of(S.fsrc_own), digest_of(S.fsrc_nb), digest_of(S.fn), digest_of(S.farea),
      digest_of(S.f_m_own), digest_of(S.f_m_nb), digest_of(S.cell_color), digest_of(S.ilu_pos),
      digest_of(S.stage_rows), digest_of(S.stage_off), digest_of(S.rcm_rank)};
  const int32_t k = (int32_t)(sizeof(d) / sizeof(d[0]));
  *n = k;
  if (digests)
    for (int32_t i = 0; i < k && i < cap; ++i) digests[i] = d[i];
  return BES_OK;
}
