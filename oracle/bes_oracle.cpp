// CPU restatement of joel-ho/BES's steady residual/update path, with a C ABI for the tests.
// TEST INFRASTRUCTURE ONLY (see bes_oracle.hpp).  Built by oracle/pyoracle.py build().
#include "bes_oracle.hpp"

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <unordered_map>

#include "linsolve.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace bor {

// Face-local vertex ordering of a tetrahedron (src/Mesh.cpp:142-146, MeshGmsh.cpp:101-106).
static const int kTetFace[4][3] = {{0, 2, 1}, {1, 2, 3}, {0, 3, 2}, {0, 1, 3}};

// MeshMath::crossProduct (src/MeshCommon.cpp:77-96): (v3 - v2) x (v1 - v2)
static void cross3(const double* a, const double* b, const double* c, double* r) {
  r[0] = (c[1] - b[1]) * (a[2] - b[2]) - (a[1] - b[1]) * (c[2] - b[2]);
  r[1] = (a[0] - b[0]) * (c[2] - b[2]) - (c[0] - b[0]) * (a[2] - b[2]);
  r[2] = (c[0] - b[0]) * (a[1] - b[1]) - (a[0] - b[0]) * (c[1] - b[1]);
}
static double dot3(const double* a, const double* b) {
  double s = 0;
  for (int d = 0; d < 3; ++d) s += a[d] * b[d];
  return s;
}
static double sq(double x) { return x * x; }

struct KeyHash {
  size_t operator()(const std::array<int64_t, 3>& k) const {
    uint64_t h = 1469598103934665603ull;
    for (int i = 0; i < 3; ++i) {
      h ^= (uint64_t)k[i] + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    }
    return (size_t)h;
  }
};

// Mesh::readGmsh tetrahedron/triangle branch + completeInitialization_ (src/Mesh.cpp:434-636),
// FaceGmshTwo::computeCenter/Normal (MeshGmsh.cpp:49-68), ElementGmshFour::computeVolume/
// computeCentroid (MeshGmsh.cpp:101-145), Element::computeAllVectorToFace / weights
// (Element.cpp:111-140), TimeStepCalculatorLocal::computeProjectedLength_ (:51-65).
static bool build_mesh(const double* X, const int64_t* tets, int64_t nc, const int64_t* btris,
                       const int32_t* btags, int64_t nb, int muscl_exact, Mesh& M, char* err) {
  std::unordered_map<std::array<int64_t, 3>, int64_t, KeyHash> key2face;
  key2face.reserve((size_t)(2 * nc + nb));
  std::vector<std::array<int64_t, 3>> fverts;
  auto make_face = [&](const int64_t* v, int kind) -> int64_t {
    const int64_t id = (int64_t)M.kind.size();
    M.kind.push_back(kind);
    fverts.push_back({v[0], v[1], v[2]});
    double c[3], S[3];
    for (int d = 0; d < 3; ++d) c[d] = (X[v[0] * 3 + d] + X[v[1] * 3 + d] + X[v[2] * 3 + d]) / 3;
    cross3(&X[v[0] * 3], &X[v[1] * 3], &X[v[2] * 3], S);
    for (int d = 0; d < 3; ++d) S[d] /= 2.0;
    double a = 0;
    for (int d = 0; d < 3; ++d) a += sq(S[d]);
    a = std::sqrt(a);
    for (int d = 0; d < 3; ++d) {
      M.center.push_back(c[d]);
      M.S.push_back(S[d]);
      M.nhat.push_back(S[d] / a);
    }
    M.area.push_back(a);
    M.owner.push_back(-1);
    M.neigh.push_back(-1);
    return id;
  };
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t* v = &btris[b * 3];
    std::array<int64_t, 3> k = {v[0], v[1], v[2]};
    std::sort(k.begin(), k.end());
    const int kind = btags[b] == 1 ? FACE_SLIP_WALL : (btags[b] == 2 ? FACE_FREESTREAM : -1);
    if (kind < 0) {
      std::snprintf(err, 256, "boundary triangle %lld has unknown tag %d", (long long)b, btags[b]);
      return false;
    }
    key2face[k] = make_face(v, kind);
  }
  M.nc = nc;
  M.cface.assign(nc * 4, -1);
  M.cadj.assign(nc * 4, -1);
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t* p = &tets[c * 4];
    for (int m = 0; m < 4; ++m) {
      int64_t v[3] = {p[kTetFace[m][0]], p[kTetFace[m][1]], p[kTetFace[m][2]]};
      std::array<int64_t, 3> k = {v[0], v[1], v[2]};
      std::sort(k.begin(), k.end());
      auto it = key2face.find(k);
      int64_t f;
      if (it != key2face.end()) {
        f = it->second;
        if (M.kind[f] != FACE_INTERNAL) {
          double out[3];
          cross3(&X[v[0] * 3], &X[v[1] * 3], &X[v[2] * 3], out);
          if (dot3(&M.S[f * 3], out) < 0) {
            for (int d = 0; d < 3; ++d) {
              M.S[f * 3 + d] = -M.S[f * 3 + d];
              M.nhat[f * 3 + d] = -M.nhat[f * 3 + d];
            }
          }
          M.owner[f] = c;
          M.neigh[f] = -1;
        } else {
          M.neigh[f] = c;
        }
      } else {
        f = make_face(v, FACE_INTERNAL);
        key2face[k] = f;
        M.owner[f] = c;
      }
      M.cface[c * 4 + m] = f;
    }
  }
  M.nf = (int64_t)M.kind.size();
  for (int64_t f = 0; f < M.nf; ++f) {
    if (M.owner[f] < 0) {
      std::snprintf(err, 256, "face %lld has no owner cell", (long long)f);
      return false;
    }
    if (M.kind[f] == FACE_INTERNAL && M.neigh[f] < 0) {
      std::snprintf(err, 256, "internal face %lld has a single cell (missing boundary triangle)",
                    (long long)f);
      return false;
    }
  }
  M.vol.assign(nc, 0);
  M.centroid.assign(nc * 3, 0);
  M.rvec.assign(nc * 12, 0);
  M.weight.assign(nc * 4, 0);
  M.plen.assign(nc * 3, 0);
  M.muscl_slot.assign(nc * 4, 0);
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t* p = &tets[c * 4];
    for (int d = 0; d < 3; ++d)
      M.centroid[c * 3 + d] =
          (X[p[0] * 3 + d] + X[p[1] * 3 + d] + X[p[2] * 3 + d] + X[p[2] * 3 + d]) / 4;
    double V = 0;
    for (int m = 0; m < 4; ++m) {
      double S[3], C[3];
      cross3(&X[p[kTetFace[m][0]] * 3], &X[p[kTetFace[m][1]] * 3], &X[p[kTetFace[m][2]] * 3], S);
      for (int d = 0; d < 3; ++d) {
        S[d] /= 2.0;
        C[d] = 0;
        for (int q = 0; q < 3; ++q) C[d] += X[p[kTetFace[m][q]] * 3 + d];
        C[d] /= 3.0;
      }
      V += dot3(C, S);
    }
    M.vol[c] = V;
    for (int m = 0; m < 4; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      for (int d = 0; d < 3; ++d)
        M.rvec[c * 12 + m * 3 + d] = M.center[f * 3 + d] - M.centroid[c * 3 + d];
    }
  }
  for (int64_t c = 0; c < nc; ++c) {
    for (int m = 0; m < 4; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      if (M.kind[f] == FACE_INTERNAL) M.cadj[c * 4 + m] = (M.owner[f] != c) ? M.owner[f] : M.neigh[f];
    }
    for (int m = 0; m < 4; ++m) {
      const int64_t a = M.cadj[c * 4 + m];
      if (a < 0) continue;
      const int64_t f = M.cface[c * 4 + m];
      double d1 = 0, d2 = 0;
      for (int d = 0; d < 3; ++d) {
        d1 += sq(M.centroid[c * 3 + d] - M.center[f * 3 + d]);
        d2 += sq(M.centroid[a * 3 + d] - M.center[f * 3 + d]);
      }
      d1 = std::sqrt(d1);
      d2 = std::sqrt(d2);
      M.weight[c * 4 + m] = d2 / (d1 + d2);
    }
    for (int m = 0; m < 4; ++m)
      for (int d = 0; d < 3; ++d) M.plen[c * 3 + d] += std::fabs(M.S[M.cface[c * 4 + m] * 3 + d]);
    for (int d = 0; d < 3; ++d) M.plen[c * 3 + d] /= 2.0;
    // Q13: Element::setSingleFace keys its face map with Face::id_ before ids are assigned
    // (src/Element.cpp:102-105 runs during readGmsh, ids are set in completeInitialization_).
    // Fresh heap objects carry id 0, so every element's map is {0 -> 3} and the lookup of
    // src/Element.cpp:185-187 returns slot 3 for face 0 and slot 0 for every other face.
    for (int m = 0; m < 4; ++m)
      M.muscl_slot[c * 4 + m] = muscl_exact ? m : (M.cface[c * 4 + m] == 0 ? 3 : 0);
  }
  return true;
}

// Mesh::readGmsh for a 2-D file (src/Mesh.cpp:235-426): boundary lines (FaceGmshOne,
// MeshGmsh.cpp:22-42: centre = midpoint, normal = (y1 - y0, x0 - x1), area = its length) are
// created first; triangle c's edges are (v0,v1), (v1,v2), (v2,v0); an edge met for the first
// time becomes an internal face with the triangle's vertex order (normal out of the triangle),
// a boundary line met by a triangle is flipped if its normal opposes the triangle's outward
// normal (MeshMath::computeTwoDimOutwardNormal, MeshCommon.cpp:60-67) and gets the triangle
// as owner, an internal edge met again gets it as neighbour.  Cells: area
// (ElementGmshTwo::computeVolume, MeshGmsh.cpp:76-82), centroid = vertex mean (:84-93), then
// the vectors, weights and projected lengths of the 3-D path over three faces; the MUSCL
// lookup (Q13) resolves face 0 to the last slot, 2.  z is read as 0 throughout.
static bool build_mesh_2d(const double* X, const int64_t* tris, int64_t nc, const int64_t* lines,
                          const int32_t* btags, int64_t nb, int muscl_exact, Mesh& M, char* err) {
  M.dim = 2;
  M.nfc = 3;
  std::unordered_map<std::array<int64_t, 3>, int64_t, KeyHash> key2face;
  key2face.reserve((size_t)(2 * nc + nb));
  auto key_of = [](int64_t a, int64_t b) {
    return std::array<int64_t, 3>{a < b ? a : b, a < b ? b : a, -1};
  };
  auto make_face = [&](int64_t a, int64_t b, int kind) -> int64_t {
    const int64_t id = (int64_t)M.kind.size();
    M.kind.push_back(kind);
    const double Sx = X[b * 3 + 1] - X[a * 3 + 1];
    const double Sy = X[a * 3] - X[b * 3];
    const double len = std::sqrt(sq(Sx) + sq(Sy));
    M.center.push_back(0.5 * (X[a * 3] + X[b * 3]));
    M.center.push_back(0.5 * (X[a * 3 + 1] + X[b * 3 + 1]));
    M.center.push_back(0.0);
    M.S.push_back(Sx);
    M.S.push_back(Sy);
    M.S.push_back(0.0);
    M.nhat.push_back(Sx / len);
    M.nhat.push_back(Sy / len);
    M.nhat.push_back(0.0);
    M.area.push_back(len);
    M.owner.push_back(-1);
    M.neigh.push_back(-1);
    return id;
  };
  for (int64_t b = 0; b < nb; ++b) {
    const int kind = btags[b] == 1 ? FACE_SLIP_WALL : (btags[b] == 2 ? FACE_FREESTREAM : -1);
    if (kind < 0) {
      std::snprintf(err, 256, "boundary line %lld has unknown tag %d", (long long)b, btags[b]);
      return false;
    }
    key2face[key_of(lines[b * 2], lines[b * 2 + 1])] = make_face(lines[b * 2], lines[b * 2 + 1], kind);
  }
  M.nc = nc;
  M.cface.assign(nc * 4, -1);
  M.cadj.assign(nc * 4, -1);
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t* p = &tris[c * 3];
    for (int m = 0; m < 3; ++m) {
      const int64_t a = p[m], b = p[(m + 1) % 3];
      const auto k = key_of(a, b);
      auto it = key2face.find(k);
      int64_t f;
      if (it == key2face.end()) {
        f = make_face(a, b, FACE_INTERNAL);
        key2face[k] = f;
        M.owner[f] = c;
      } else {
        f = it->second;
        if (M.kind[f] != FACE_INTERNAL) {
          const double ox = X[b * 3 + 1] - X[a * 3 + 1];
          const double oy = -X[b * 3] + X[a * 3];
          if (M.S[f * 3] * ox + M.S[f * 3 + 1] * oy < 0)
            for (int d = 0; d < 2; ++d) {
              M.S[f * 3 + d] = -M.S[f * 3 + d];
              M.nhat[f * 3 + d] = -M.nhat[f * 3 + d];
            }
          M.owner[f] = c;
          M.neigh[f] = -1;
        } else {
          M.neigh[f] = c;
        }
      }
      M.cface[c * 4 + m] = f;
    }
  }
  M.nf = (int64_t)M.kind.size();
  for (int64_t f = 0; f < M.nf; ++f) {
    if (M.owner[f] < 0) {
      std::snprintf(err, 256, "face %lld has no owner cell", (long long)f);
      return false;
    }
    if (M.kind[f] == FACE_INTERNAL && M.neigh[f] < 0) {
      std::snprintf(err, 256, "internal edge %lld has a single cell (missing boundary line)",
                    (long long)f);
      return false;
    }
  }
  M.vol.assign(nc, 0);
  M.centroid.assign(nc * 3, 0);
  M.rvec.assign(nc * 12, 0);
  M.weight.assign(nc * 4, 0);
  M.plen.assign(nc * 3, 0);
  M.muscl_slot.assign(nc * 4, 0);
  for (int64_t c = 0; c < nc; ++c) {
    const double* v0 = &X[tris[c * 3] * 3];
    const double* v1 = &X[tris[c * 3 + 1] * 3];
    const double* v2 = &X[tris[c * 3 + 2] * 3];
    M.vol[c] = 0.5 * std::fabs((v0[0] - v1[0]) * (v2[1] - v1[1]) - (v2[0] - v1[0]) * (v0[1] - v1[1]));
    for (int d = 0; d < 2; ++d) M.centroid[c * 3 + d] = (v0[d] + v1[d] + v2[d]) / 3;
    for (int m = 0; m < 3; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      for (int d = 0; d < 2; ++d)
        M.rvec[c * 12 + m * 3 + d] = M.center[f * 3 + d] - M.centroid[c * 3 + d];
    }
  }
  for (int64_t c = 0; c < nc; ++c) {
    for (int m = 0; m < 3; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      if (M.kind[f] == FACE_INTERNAL) M.cadj[c * 4 + m] = (M.owner[f] != c) ? M.owner[f] : M.neigh[f];
    }
    for (int m = 0; m < 3; ++m) {
      const int64_t a = M.cadj[c * 4 + m];
      if (a < 0) continue;
      const int64_t f = M.cface[c * 4 + m];
      double d1 = 0, d2 = 0;
      for (int d = 0; d < 2; ++d) {
        d1 += sq(M.centroid[c * 3 + d] - M.center[f * 3 + d]);
        d2 += sq(M.centroid[a * 3 + d] - M.center[f * 3 + d]);
      }
      d1 = std::sqrt(d1);
      d2 = std::sqrt(d2);
      M.weight[c * 4 + m] = d2 / (d1 + d2);
    }
    for (int m = 0; m < 3; ++m)
      for (int d = 0; d < 2; ++d) M.plen[c * 3 + d] += std::fabs(M.S[M.cface[c * 4 + m] * 3 + d]);
    for (int d = 0; d < 2; ++d) M.plen[c * 3 + d] /= 2.0;
    for (int m = 0; m < 3; ++m)
      M.muscl_slot[c * 4 + m] = muscl_exact ? m : (M.cface[c * 4 + m] == 0 ? 2 : 0);
    M.muscl_slot[c * 4 + 3] = -1;
  }
  return true;
}

struct Oracle {
  Mesh M;
  Gas g;
  Options o;
  double Pinf[6];
  int threads = 1;
  std::vector<int64_t> cface_sorted;  // per cell, local face indices in increasing face id
  // explicit state
  std::vector<double> Un, Uk, dt, G, phi, F, R;
  double global_dt = 0;
  // implicit
  besla::BlockCsr A;
  std::vector<int64_t> blk_own_own, blk_own_nb, blk_nb_own, blk_nb_nb;  // per face block ids
  std::vector<double> JL, JR, rhs, dW;
  std::vector<int64_t> ilu_order;
  std::vector<int64_t> ilu_domain;  // optional subdomain per cell (block Jacobi over them)
  double cfl_actual = 0;
  double maxres[5] = {0, 0, 0, 0, 0}, maxres_old[5] = {0, 0, 0, 0, 0};
  int step_count = 0;
  int64_t solver_step = 0;  // iteration / pseudo-time step index (freestream ramp)
  int last_lin_iters = 0;
  double last_lin_err = 0;
  char err[256] = {0};
};

// Config::getFreestreamPrimitiveVariables (src/Config.cpp:688-706)
static void set_freestream_for_step(Oracle& O, int64_t t) {
  O.Pinf[0] = 1.0;
  for (int d = 0; d < 3; ++d) O.Pinf[1 + d] = O.o.mach[d];
  O.Pinf[4] = 1.0 / O.o.gamma;
  O.Pinf[5] = 1.0 / (O.o.gamma * O.o.gas_constant);
  if (O.o.fs_ramp > 0 && t < O.o.fs_ramp)
    for (int d = 0; d < 3; ++d)
      O.Pinf[1 + d] = O.o.mach[d] * (O.o.fs_frac + static_cast<double>(t) /
                                                       static_cast<double>(O.o.fs_ramp) *
                                                       (1 - O.o.fs_frac));
}

static void init_state(Oracle& O) {
  // Config::initializePostMesh freestream primitives (src/Config.cpp:480-488)
  set_freestream_for_step(O, 0);
  double U[5];
  O.g.conserved(O.Pinf, U);  // setUniversalInitialCondition (SolverExplicit.cpp:233-257)
  O.Un.assign(O.M.nc * 5, 0);
  for (int64_t c = 0; c < O.M.nc; ++c)
    for (int v = 0; v < 5; ++v) O.Un[c * 5 + v] = U[v];
  O.Uk = O.Un;
}

// TimeStepCalculatorLocal/Global::computeAllTimeStep (src/TimeStepCalculatorLocal.cpp:67-93,
// src/TimeStepCalculatorGlobal.cpp:64-98)
static void compute_dt(Oracle& O, const double* U, double cfl) {
  const Mesh& M = O.M;
  O.dt.resize(M.nc);
#pragma omp parallel for num_threads(O.threads)
  for (int64_t c = 0; c < M.nc; ++c) {
    const double* u = &U[c * 5];
    double spec = 0.0;
    const double cs = O.g.sound_speed_U(u);
    for (int d = 0; d < 3; ++d) {
      const double vel = std::fabs(O.g.velocity(u, d));
      spec += (cs + vel) * M.plen[c * 3 + d];
    }
    O.dt[c] = cfl * M.vol[c] / spec;
  }
  if (!O.o.local_dt) {
    double mn = O.dt[0];
    for (int64_t c = 1; c < M.nc; ++c) mn = O.dt[c] < mn ? O.dt[c] : mn;
    O.global_dt = mn;
    std::fill(O.dt.begin(), O.dt.end(), mn);
  }
}

// GradientGreenGauss::computeGradient (src/GradientGreenGauss.cpp:21-135)
static void compute_gradient(Oracle& O, const double* U) {
  const Mesh& M = O.M;
  O.G.assign(M.nc * 15, 0);
#pragma omp parallel for num_threads(O.threads)
  for (int64_t c = 0; c < M.nc; ++c) {
    double* G = &O.G[c * 15];
    const double* ui = &U[c * 5];
    for (int m = 0; m < M.nfc; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      const double* S = &M.S[f * 3];
      const int64_t nb = M.cadj[c * 4 + m];
      const double w = M.weight[c * 4 + m];
      for (int v = 0; v < 5; ++v)
        for (int d = 0; d < 3; ++d) {
          if (nb < 0)
            G[v * 3 + d] += S[d] * (ui[v]);
          else if (M.owner[f] == c)
            G[v * 3 + d] += S[d] * (w * ui[v] + (1 - w) * U[nb * 5 + v]);
          else
            G[v * 3 + d] -= S[d] * (w * ui[v] + (1 - w) * U[nb * 5 + v]);
        }
      if (M.kind[f] == FACE_SLIP_WALL) {
        const double* n = &M.nhat[f * 3];
        double vn = 0;
        for (int d = 0; d < 3; ++d) vn += ui[1 + d] * n[d];
        double t[3];
        for (int d = 0; d < 3; ++d) t[d] = ui[1 + d] - vn * n[d];
        for (int a = 0; a < 3; ++a)
          for (int d = 0; d < 3; ++d) G[(1 + a) * 3 + d] += (t[a] * S[d] - ui[1 + a] * S[d]);
      }
    }
    for (int q = 0; q < 15; ++q) G[q] /= M.vol[c];
  }
}

// LimiterVenkatakrishnan::computeLimiterTerm / computeFaceLimiter_
// (src/LimiterVenkatakrishnan.cpp:21-128)
static double venkat_face(double dmin, double dmax, double d2, double eps) {
  if (d2 > 0)
    return (1 / d2) * ((dmax * dmax + eps * eps) * d2 + 2.0 * d2 * d2 * dmax) /
           (dmax * dmax + 2.0 * d2 * d2 + dmax * d2 + eps * eps);
  if (d2 < 0)
    return (1 / d2) * ((dmin * dmin + eps * eps) * d2 + 2.0 * d2 * d2 * dmin) /
           (dmin * dmin + 2.0 * d2 * d2 + dmin * d2 + eps * eps);
  return 1.0;
}
static void compute_limiter(Oracle& O, const double* U) {
  const Mesh& M = O.M;
  O.phi.assign(M.nc * 5, 0);
#pragma omp parallel for num_threads(O.threads)
  for (int64_t c = 0; c < M.nc; ++c) {
    const double len = std::pow(M.vol[c], 1.0 / M.dim);
    const double eps = std::pow(O.o.venkat_k * len, 3.0 / 2.0);
    for (int v = 0; v < 5; ++v) {
      const double ui = U[c * 5 + v];
      double dmin = ui, dmax = ui;
      for (int m = 0; m < 4; ++m) {
        const int64_t nb = M.cadj[c * 4 + m];
        if (nb < 0) continue;
        const double x = U[nb * 5 + v];
        dmin = (x < dmin) ? x : dmin;
        dmax = (x > dmax) ? x : dmax;
      }
      dmin -= ui;
      dmax -= ui;
      double lim = 1.0;
      for (int m = 0; m < 4; ++m) {
        if (M.cadj[c * 4 + m] < 0) continue;
        double d2 = 0;
        for (int d = 0; d < 3; ++d) d2 += O.G[c * 15 + v * 3 + d] * M.rvec[c * 12 + m * 3 + d];
        d2 /= 2.0;
        const double p = venkat_face(dmin, dmax, d2, eps);
        lim = p < lim ? p : lim;
      }
      O.phi[c * 5 + v] = lim;
    }
  }
}

// Solver::computeFaceConservedVariable_ (src/Solver.cpp:69-121), side of cell c at local face m
static void muscl_side(const Oracle& O, const double* U, int64_t c, int m, double* out) {
  const int slot = O.M.muscl_slot[c * 4 + m];
  const double* r = &O.M.rvec[c * 12 + slot * 3];
  for (int v = 0; v < 5; ++v) {
    const double lim = O.phi[c * 5 + v];
    double x = U[c * 5 + v];
    for (int d = 0; d < 3; ++d) x += lim * O.G[c * 15 + v * 3 + d] * r[d];
    out[v] = x;
  }
}
static int local_index(const Mesh& M, int64_t c, int64_t f) {
  for (int m = 0; m < 4; ++m)
    if (M.cface[c * 4 + m] == f) return m;
  return -1;
}
static void face_states(const Oracle& O, const double* U, int64_t f, double* UL, double* UR) {
  const Mesh& M = O.M;
  const int64_t o = M.owner[f];
  muscl_side(O, U, o, local_index(M, o, f), UL);
  const int64_t nb = M.neigh[f];
  if (nb >= 0)
    muscl_side(O, U, nb, local_index(M, nb, f), UR);
  else
    for (int v = 0; v < 5; ++v) UR[v] = 0;
}

static void face_flux(const Oracle& O, int64_t f, const double* UL, const double* UR, double* Ff) {
  const double* n = &O.M.nhat[f * 3];
  switch (O.M.kind[f]) {
    case FACE_INTERNAL: flux_roe(O.g, O.o.harten, UL, UR, n, Ff); break;
    case FACE_FREESTREAM: flux_freestream(O.g, UL, O.Pinf, n, Ff); break;
    case FACE_SLIP_WALL: flux_slipwall(O.g, UL, n, Ff); break;
  }
}

// Face loop of SolverExplicit::timeStep_ (src/SolverExplicit.cpp:285-344): per-face flux, then
// R_c = sum over the cell's faces, in increasing face id (the order a single thread adds).
static void compute_residual(Oracle& O, const double* U) {
  const Mesh& M = O.M;
  O.F.assign(M.nf * 5, 0);
#pragma omp parallel for num_threads(O.threads)
  for (int64_t f = 0; f < M.nf; ++f) {
    double UL[5], UR[5];
    face_states(O, U, f, UL, UR);
    face_flux(O, f, UL, UR, &O.F[f * 5]);
  }
  O.R.assign(M.nc * 5, 0);
#pragma omp parallel for num_threads(O.threads)
  for (int64_t c = 0; c < M.nc; ++c) {
    for (int q = 0; q < M.nfc; ++q) {
      const int m = (int)O.cface_sorted[c * 4 + q];
      const int64_t f = M.cface[c * 4 + m];
      for (int v = 0; v < 5; ++v) {
        if (M.owner[f] == c)
          O.R[c * 5 + v] += O.F[f * 5 + v] * M.area[f];
        else
          O.R[c * 5 + v] -= O.F[f * 5 + v] * M.area[f];
      }
    }
  }
}

static void norms(const Mesh& M, const std::vector<double>& R, double* out10) {
  for (int v = 0; v < 5; ++v) {
    double s = 0, mx = 0;
    for (int64_t c = 0; c < M.nc; ++c) {
      const double a = R[c * 5 + v];
      s += a * a;
      mx = std::fabs(a) > mx ? std::fabs(a) : mx;
    }
    out10[v] = std::sqrt(s);
    out10[5 + v] = mx;
  }
}

// SolverExplicit::timeStep_ (src/SolverExplicit.cpp:259-393)
static void explicit_iteration(Oracle& O, double* norms10) {
  set_freestream_for_step(O, O.solver_step++);
  compute_dt(O, O.Un.data(), O.o.cfl);
  const Mesh& M = O.M;
  for (int k = 0; k < O.o.n_stage; ++k) {
    const double* U = (k == 0) ? O.Un.data() : O.Uk.data();
    compute_gradient(O, U);
    compute_limiter(O, U);
    compute_residual(O, U);
    const double a = O.o.alpha[k];
#pragma omp parallel for num_threads(O.threads)
    for (int64_t c = 0; c < M.nc; ++c)
      for (int v = 0; v < 5; ++v)
        O.Uk[c * 5 + v] = O.Un[c * 5 + v] - (a * O.dt[c] / M.vol[c]) * O.R[c * 5 + v];
  }
  if (norms10) norms(M, O.R, norms10);
  O.Un.swap(O.Uk);
  O.Uk = O.Un;
}

// ---------------------------------------------------------------------------------
// implicit path (src/SolverImplicit.cpp:293-550)
// ---------------------------------------------------------------------------------
static void jac_kind(const Oracle& O, int kind, const double* n, const double* U1L,
                     const double* U1R, double* JLo, double* JRo) {
  switch (kind) {
    case FACE_INTERNAL: {
      Dual<10> L[5], R[5], Fd[5];
      for (int v = 0; v < 5; ++v) {
        L[v] = Dual<10>(U1L[v]);
        L[v].d[v] = 1.0;
        R[v] = Dual<10>(U1R[v]);
        R[v].d[5 + v] = 1.0;
      }
      flux_roe(O.g, O.o.harten, L, R, n, Fd);
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) {
          JLo[r * 5 + c] = Fd[r].d[c];
          JRo[r * 5 + c] = Fd[r].d[5 + c];
        }
      break;
    }
    case FACE_FREESTREAM: {
      Dual<5> L[5], Fd[5];
      for (int v = 0; v < 5; ++v) {
        L[v] = Dual<5>(U1L[v]);
        L[v].d[v] = 1.0;
      }
      flux_freestream(O.g, L, O.Pinf, n, Fd);
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) JLo[r * 5 + c] = Fd[r].d[c];
      break;
    }
    case FACE_SLIP_WALL: {
      Dual<5> L[5], Fd[5];
      for (int v = 0; v < 5; ++v) {
        L[v] = Dual<5>(U1L[v]);
        L[v].d[v] = 1.0;
      }
      flux_slipwall(O.g, L, n, Fd);
      for (int r = 0; r < 5; ++r)
        for (int c = 0; c < 5; ++c) JLo[r * 5 + c] = Fd[r].d[c];
      break;
    }
  }
}

// CoefficientMatrix::initialize pattern (src/CoefficientMatrix.cpp:114-164): block row per
// cell, diagonal block first, then one block per adjacent cell in local face order.
static void build_pattern(Oracle& O) {
  const Mesh& M = O.M;
  besla::BlockCsr& A = O.A;
  A.n = M.nc;
  A.row.assign(M.nc + 1, 0);
  for (int64_t c = 0; c < M.nc; ++c) {
    int cnt = 1;
    for (int m = 0; m < 4; ++m) cnt += M.cadj[c * 4 + m] >= 0;
    A.row[c + 1] = A.row[c] + cnt;
  }
  A.col.assign(A.row[M.nc], 0);
  A.diag.assign(M.nc, 0);
  std::vector<int64_t> slot_of(M.nc * 4, -1);
  for (int64_t c = 0; c < M.nc; ++c) {
    int64_t k = A.row[c];
    A.diag[c] = k;
    A.col[k++] = c;
    for (int m = 0; m < 4; ++m) {
      const int64_t a = M.cadj[c * 4 + m];
      if (a < 0) continue;
      slot_of[c * 4 + m] = k;
      A.col[k++] = a;
    }
  }
  A.val.assign(A.row[M.nc] * 25, 0.0);
  O.blk_own_own.assign(M.nf, -1);
  O.blk_own_nb.assign(M.nf, -1);
  O.blk_nb_own.assign(M.nf, -1);
  O.blk_nb_nb.assign(M.nf, -1);
  for (int64_t f = 0; f < M.nf; ++f) {
    const int64_t o = M.owner[f];
    O.blk_own_own[f] = A.diag[o];
    const int64_t nb = M.neigh[f];
    if (nb < 0) continue;
    O.blk_nb_nb[f] = A.diag[nb];
    O.blk_own_nb[f] = slot_of[o * 4 + local_index(M, o, f)];
    O.blk_nb_own[f] = slot_of[nb * 4 + local_index(M, nb, f)];
  }
  if (O.ilu_order.empty()) {
    O.ilu_order.resize(M.nc);
    for (int64_t c = 0; c < M.nc; ++c) O.ilu_order[c] = c;
  }
}

static double implicit_cfl_for_step(const Oracle& O) {
  if (O.o.ramp_steps > 0) {
    const int k = O.step_count;
    if (k >= O.o.ramp_steps - 1 || O.o.ramp_steps == 1) return O.o.ramp_cfl1;
    const double t = (double)k / (double)(O.o.ramp_steps - 1);
    return O.o.ramp_cfl0 * std::pow(O.o.ramp_cfl1 / O.o.ramp_cfl0, t);
  }
  return O.cfl_actual;
}

// SolverImplicit::timeStep_ (src/SolverImplicit.cpp:293-345), computeFaceFluxes_ (:358-507),
// updateSolution_ (:509-528), adaptCourantNum_ (:530-550)
static void implicit_step(Oracle& O, double* hist) {
  const Mesh& M = O.M;
  // resetSystemOfEquation_ (:347-356)
  O.rhs.assign(M.nc * 5, 0.0);
  O.dW.assign(M.nc * 5, 0.0);
  std::fill(O.A.val.begin(), O.A.val.end(), 0.0);
  for (int64_t c = 0; c < M.nc; ++c)
    for (int r = 0; r < 5; ++r) O.A.val[O.A.diag[c] * 25 + r * 6] += 1;
  for (int v = 0; v < 5; ++v) {
    O.maxres_old[v] = O.maxres[v];
    O.maxres[v] = 0;
  }
  const double cfl = implicit_cfl_for_step(O);
  set_freestream_for_step(O, O.solver_step++);
  const double* U = O.Un.data();
  compute_dt(O, U, cfl);
  compute_gradient(O, U);
  compute_limiter(O, U);
  // per-face second-order flux and first-order Jacobians
  O.F.assign(M.nf * 5, 0);
  O.JL.assign(M.nf * 25, 0);
  O.JR.assign(M.nf * 25, 0);
#pragma omp parallel for num_threads(O.threads)
  for (int64_t f = 0; f < M.nf; ++f) {
    double UL[5], UR[5];
    face_states(O, U, f, UL, UR);
    face_flux(O, f, UL, UR, &O.F[f * 5]);
    double U1L[5], U1R[5];
    const int64_t o = M.owner[f], nb = M.neigh[f];
    for (int v = 0; v < 5; ++v) {
      U1L[v] = U[o * 5 + v];
      U1R[v] = nb >= 0 ? U[nb * 5 + v] : 0.0;
    }
    jac_kind(O, M.kind[f], &M.nhat[f * 3], U1L, U1R, &O.JL[f * 25], &O.JR[f * 25]);
  }
  // Assembly, per cell in increasing face id: identical to the face loop's sequence of
  // atomic adds at one thread.  Every block is added jacobian_repeat times (Q9: once per
  // conserved variable, 5 in 3-D and 4 in 2-D).
  const int rep = O.o.jacobian_repeat;
#pragma omp parallel for num_threads(O.threads)
  for (int64_t c = 0; c < M.nc; ++c) {
    for (int q = 0; q < M.nfc; ++q) {
      const int m = (int)O.cface_sorted[c * 4 + q];
      const int64_t f = M.cface[c * 4 + m];
      const int64_t o = M.owner[f], nb = M.neigh[f];
      const double A_f = M.area[f];
      if (o == c) {
        const double mL = O.dt[o] / M.vol[o] * A_f;
        for (int v = 0; v < 5; ++v) O.rhs[c * 5 + v] -= mL * O.F[f * 5 + v];
        double* B = &O.A.val[O.blk_own_own[f] * 25];
        for (int r = 0; r < rep; ++r)
          for (int q2 = 0; q2 < 25; ++q2) B[q2] += mL * O.JL[f * 25 + q2];
        if (nb >= 0) {
          double* B2 = &O.A.val[O.blk_own_nb[f] * 25];
          for (int r = 0; r < rep; ++r)
            for (int q2 = 0; q2 < 25; ++q2) B2[q2] += mL * O.JR[f * 25 + q2];
        }
      } else {
        const double mR = O.dt[nb] / M.vol[nb] * A_f;
        for (int v = 0; v < 5; ++v) O.rhs[c * 5 + v] += O.dt[nb] / M.vol[nb] * A_f * O.F[f * 5 + v];
        double* B = &O.A.val[O.blk_nb_own[f] * 25];
        double* B2 = &O.A.val[O.blk_nb_nb[f] * 25];
        for (int r = 0; r < rep; ++r)
          for (int q2 = 0; q2 < 25; ++q2) {
            B[q2] += -mR * O.JL[f * 25 + q2];
            B2[q2] += -mR * O.JR[f * 25 + q2];
          }
      }
    }
  }
  besla::Preconditioner P;
  P.dom = O.ilu_domain;
  if (O.o.lin_precond == 1)
    P.setup_ilu0(O.A, O.ilu_order);
  else
    P.setup_jacobi(O.A);
  besla::GmresResult gr =
      besla::gmres(O.A, P, O.rhs.data(), O.dW.data(), O.o.lin_restart, O.o.lin_maxiter, O.o.lin_tol);
  O.last_lin_iters = gr.iterations;
  O.last_lin_err = gr.rel_residual;
  for (int64_t c = 0; c < M.nc; ++c)
    for (int v = 0; v < 5; ++v) {
      O.Un[c * 5 + v] += O.dW[c * 5 + v];
      const double a = std::fabs(O.rhs[c * 5 + v]);
      O.maxres[v] = a > O.maxres[v] ? a : O.maxres[v];
    }
  if (hist) {
    for (int v = 0; v < 5; ++v) {
      double s = 0;
      for (int64_t c = 0; c < M.nc; ++c) s += O.rhs[c * 5 + v] * O.rhs[c * 5 + v];
      hist[v] = std::sqrt(s);
      hist[5 + v] = O.maxres[v];
    }
    hist[10] = cfl;
    // L2 of the unscaled residual R = sum(+-F A), summed per cell in increasing face id
    double r2[5] = {0, 0, 0, 0, 0};
    for (int64_t c = 0; c < M.nc; ++c) {
      double R[5] = {0, 0, 0, 0, 0};
      for (int q = 0; q < M.nfc; ++q) {
        const int m = (int)O.cface_sorted[c * 4 + q];
        const int64_t f = M.cface[c * 4 + m];
        for (int v = 0; v < 5; ++v) {
          if (M.owner[f] == c)
            R[v] += O.F[f * 5 + v] * M.area[f];
          else
            R[v] -= O.F[f * 5 + v] * M.area[f];
        }
      }
      for (int v = 0; v < 5; ++v) r2[v] += R[v] * R[v];
    }
    for (int v = 0; v < 5; ++v) hist[12 + v] = std::sqrt(r2[v]);
  }
  if (O.o.ramp_steps <= 0 && O.o.cfl_max > O.o.cfl) {  // adaptCourantNum_
    const int idx = (O.maxres_old[0] > O.maxres[0]) ? 1 : 0;
    O.cfl_actual *= std::pow(O.maxres_old[0] / O.maxres[0], O.o.cfl_exp[idx]);
    O.cfl_actual = std::max(O.o.cfl, O.cfl_actual);
    O.cfl_actual = std::min(O.o.cfl_max, O.cfl_actual);
  }
  if (hist) hist[11] = O.cfl_actual;
  ++O.step_count;
}

}  // namespace bor

// =================================================================================
// C ABI (ctypes)
// =================================================================================
extern "C" {

struct bor_options {
  int32_t solver, local_dt, n_stage, muscl_exact;
  int32_t jacobian_repeat, lin_precond, lin_restart, lin_maxiter;
  int32_t ramp_steps, threads, pad0, pad1;
  double cfl, cfl_max, cfl_exp0, cfl_exp1;
  double alpha[8];
  double venkat_k, harten, gas_constant, gamma;
  double mach[3];
  double lin_tol, ramp_cfl0, ramp_cfl1;
  int32_t fs_ramp, pad2;
  double fs_frac;
};

void* bor_create(const double* nodes, int64_t nv, const int64_t* tets, int64_t nc,
                 const int64_t* btris, const int32_t* btags, int64_t nb, int32_t dim,
                 const bor_options* op, char* errbuf) {
  (void)nv;
  bor::Oracle* O = new bor::Oracle();
  bor::Options& o = O->o;
  o.solver = op->solver;
  o.local_dt = op->local_dt;
  o.n_stage = op->n_stage;
  o.muscl_exact = op->muscl_exact;
  // 0: the reference's count, once per conserved variable (src/SolverImplicit.cpp:425-502)
  o.jacobian_repeat = op->jacobian_repeat > 0 ? op->jacobian_repeat : (dim == 2 ? 4 : 5);
  o.lin_precond = op->lin_precond;
  o.lin_restart = op->lin_restart;
  o.lin_maxiter = op->lin_maxiter;
  o.ramp_steps = op->ramp_steps;
  o.cfl = op->cfl;
  o.cfl_max = op->cfl_max;
  o.cfl_exp[0] = op->cfl_exp0;
  o.cfl_exp[1] = op->cfl_exp1;
  for (int i = 0; i < 8; ++i) o.alpha[i] = op->alpha[i];
  o.venkat_k = op->venkat_k;
  o.harten = op->harten;
  o.gas_constant = op->gas_constant;
  o.gamma = op->gamma;
  for (int d = 0; d < 3; ++d) o.mach[d] = op->mach[d];
  o.lin_tol = op->lin_tol;
  o.ramp_cfl0 = op->ramp_cfl0;
  o.ramp_cfl1 = op->ramp_cfl1;
  o.fs_ramp = op->fs_ramp;
  o.fs_frac = op->fs_frac;
  O->threads = op->threads > 0 ? op->threads : 1;
  O->g.init(o.gas_constant, o.gamma);
  const bool ok = dim == 2 ? bor::build_mesh_2d(nodes, tets, nc, btris, btags, nb,
                                                 o.muscl_exact, O->M, O->err)
                           : bor::build_mesh(nodes, tets, nc, btris, btags, nb, o.muscl_exact,
                                             O->M, O->err);
  if (!ok) {
    if (errbuf) std::snprintf(errbuf, 256, "%s", O->err);
    delete O;
    return nullptr;
  }
  // per cell, the local faces in increasing face id (the order the reference's face loop adds
  // them to a cell's residual); the empty slot of a triangle stays last
  const int nfc = O->M.nfc;
  O->cface_sorted.resize(nc * 4);
  for (int64_t c = 0; c < nc; ++c) {
    int64_t idx[4] = {0, 1, 2, 3};
    std::sort(idx, idx + nfc, [&](int64_t a, int64_t b) {
      return O->M.cface[c * 4 + a] < O->M.cface[c * 4 + b];
    });
    for (int q = 0; q < 4; ++q) O->cface_sorted[c * 4 + q] = idx[q];
  }
  bor::init_state(*O);
  O->cfl_actual = o.cfl;
  return O;
}

void bor_destroy(void* h) { delete static_cast<bor::Oracle*>(h); }

void bor_sizes(void* h, int64_t* out) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  out[0] = O->M.nc;
  out[1] = O->M.nf;
}

// Geometry in reference numbering.
void bor_geometry(void* h, double* vol, double* centroid, double* rvec, double* weight,
                  int64_t* cface, int64_t* cadj, double* S, double* nhat, double* area,
                  double* center, int64_t* owner, int64_t* neigh, int64_t* kind, int64_t* slot) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  const bor::Mesh& M = O->M;
  std::memcpy(vol, M.vol.data(), M.nc * 8);
  std::memcpy(centroid, M.centroid.data(), M.nc * 24);
  std::memcpy(rvec, M.rvec.data(), M.nc * 96);
  std::memcpy(weight, M.weight.data(), M.nc * 32);
  std::memcpy(cface, M.cface.data(), M.nc * 32);
  std::memcpy(cadj, M.cadj.data(), M.nc * 32);
  std::memcpy(S, M.S.data(), M.nf * 24);
  std::memcpy(nhat, M.nhat.data(), M.nf * 24);
  std::memcpy(area, M.area.data(), M.nf * 8);
  std::memcpy(center, M.center.data(), M.nf * 24);
  std::memcpy(owner, M.owner.data(), M.nf * 8);
  std::memcpy(neigh, M.neigh.data(), M.nf * 8);
  for (int64_t f = 0; f < M.nf; ++f) kind[f] = M.kind[f];
  for (int64_t q = 0; q < M.nc * 4; ++q) slot[q] = M.muscl_slot[q];
}

void bor_set_state(void* h, const double* U) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  std::memcpy(O->Un.data(), U, O->M.nc * 40);
  O->Uk = O->Un;
}
void bor_get_state(void* h, double* U) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  std::memcpy(U, O->Un.data(), O->M.nc * 40);
}

// Operators at the current state: dt (at cfl), gradients, limiters, MUSCL face states,
// per-face fluxes (per unit area) and the residual R.
void bor_operators(void* h, double cfl, double* dt, double* G, double* phi, double* UL,
                   double* UR, double* F, double* R) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  const bor::Mesh& M = O->M;
  const double* U = O->Un.data();
  bor::set_freestream_for_step(*O, O->solver_step);  // the freestream of the next step
  bor::compute_dt(*O, U, cfl);
  bor::compute_gradient(*O, U);
  bor::compute_limiter(*O, U);
  bor::compute_residual(*O, U);
  if (dt) std::memcpy(dt, O->dt.data(), M.nc * 8);
  if (G) std::memcpy(G, O->G.data(), M.nc * 120);
  if (phi) std::memcpy(phi, O->phi.data(), M.nc * 40);
  if (F) std::memcpy(F, O->F.data(), M.nf * 40);
  if (R) std::memcpy(R, O->R.data(), M.nc * 40);
  if (UL || UR)
    for (int64_t f = 0; f < M.nf; ++f) {
      double l[5], r[5];
      bor::face_states(*O, U, f, l, r);
      if (UL) std::memcpy(&UL[f * 5], l, 40);
      if (UR) std::memcpy(&UR[f * 5], r, 40);
    }
}

// n explicit iterations; hist [n*10] = L2[5], Linf[5] of the last stage's R.
void bor_explicit_run(void* h, int64_t n, double* hist) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  for (int64_t i = 0; i < n; ++i) bor::explicit_iteration(*O, hist ? &hist[i * 10] : nullptr);
}

void bor_set_ilu_domain(void* h, const int64_t* dom) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  if (dom)
    O->ilu_domain.assign(dom, dom + O->M.nc);
  else
    O->ilu_domain.clear();
}

void bor_set_ilu_order(void* h, const int64_t* order) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  O->ilu_order.assign(order, order + O->M.nc);
}

// n implicit steps; hist [n*19] = L2[5] and max[5] of the Dt/V-scaled RHS, CFL used,
// CFL after adaptation, linear iterations, linear relative residual, L2[5] of R.
void bor_implicit_run(void* h, int64_t n, double* hist) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  if (O->A.n == 0) bor::build_pattern(*O);
  for (int64_t i = 0; i < n; ++i) {
    double loc[17];
    bor::implicit_step(*O, loc);
    if (hist) {
      std::memcpy(&hist[i * 19], loc, 12 * sizeof(double));
      hist[i * 19 + 12] = O->last_lin_iters;
      hist[i * 19 + 13] = O->last_lin_err;
      for (int v = 0; v < 5; ++v) hist[i * 19 + 14 + v] = loc[12 + v];
    }
  }
}

// Assemble (without solving) the implicit system at the current state with the given CFL.
// rhs [nc*5]; blocks in the pattern's order [nblk*25]; rowptr [nc+1], col [nblk].
int64_t bor_implicit_assemble(void* h, double cfl, double* rhs, double* vals, int64_t* rowptr,
                              int64_t* col) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  if (O->A.n == 0) bor::build_pattern(*O);
  const int32_t ramp = O->o.ramp_steps;
  const double keep = O->cfl_actual;
  O->o.ramp_steps = 0;
  O->cfl_actual = cfl;
  // run the assembly part of a step without touching the state
  std::vector<double> U0 = O->Un;
  double mr[5], mro[5];
  std::memcpy(mr, O->maxres, sizeof(mr));
  std::memcpy(mro, O->maxres_old, sizeof(mro));
  const int lp = O->o.lin_maxiter;
  O->o.lin_maxiter = 0;
  double loc[17];
  bor::implicit_step(*O, loc);
  O->o.lin_maxiter = lp;
  O->Un = U0;
  --O->solver_step;
  std::memcpy(O->maxres, mr, sizeof(mr));
  std::memcpy(O->maxres_old, mro, sizeof(mro));
  O->o.ramp_steps = ramp;
  O->cfl_actual = keep;
  --O->step_count;
  const int64_t nblk = O->A.row[O->M.nc];
  if (rhs) std::memcpy(rhs, O->rhs.data(), O->M.nc * 40);
  if (vals) std::memcpy(vals, O->A.val.data(), nblk * 200);
  if (rowptr) std::memcpy(rowptr, O->A.row.data(), (O->M.nc + 1) * 8);
  if (col) std::memcpy(col, O->A.col.data(), nblk * 8);
  return nblk;
}

// Known-answer entry points: kind 0 Roe, 1 slip wall, 2 freestream (UR unused; Pinf from the
// handle's options).  F [n*5]; JL, JR [n*25] (JR only for Roe; may be null).
void bor_flux_batch(void* h, int32_t kind, int64_t n, const double* UL, const double* UR,
                    const double* nhat, double* F, double* JL, double* JR) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  for (int64_t i = 0; i < n; ++i) {
    const double* nn = &nhat[i * 3];
    if (kind == 0)
      bor::flux_roe(O->g, O->o.harten, &UL[i * 5], &UR[i * 5], nn, &F[i * 5]);
    else if (kind == 1)
      bor::flux_slipwall(O->g, &UL[i * 5], nn, &F[i * 5]);
    else
      bor::flux_freestream(O->g, &UL[i * 5], O->Pinf, nn, &F[i * 5]);
    if (JL) {
      double jr[25];
      const double zero[5] = {0, 0, 0, 0, 0};
      const int k = kind == 0 ? bor::FACE_INTERNAL : (kind == 1 ? bor::FACE_SLIP_WALL : bor::FACE_FREESTREAM);
      bor::jac_kind(*O, k, nn, &UL[i * 5], kind == 0 ? &UR[i * 5] : zero, &JL[i * 25],
                    JR ? &JR[i * 25] : jr);
    }
  }
}

void bor_pinf(void* h, double* out6) {
  bor::Oracle* O = static_cast<bor::Oracle*>(h);
  for (int i = 0; i < 6; ++i) out6[i] = O->Pinf[i];
}

}  // extern "C"
