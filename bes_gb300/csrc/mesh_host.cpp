// Host-side mesh pre-processing (runs once per context).
//
// Face discovery reproduces Mesh::readGmsh (src/Mesh.cpp:95-558 of joel-ho/BES) with an
// open-addressing hash table instead of the reference's string-keyed std::map: faces are
// keyed by their sorted vertex ids, boundary triangles are created first in file order, a
// tetrahedron's faces follow the local ordering {0,2,1},{1,2,3},{0,3,2},{0,1,3}, the first
// tetrahedron that meets a face owns it, and boundary normals are flipped to point out of
// their owner.  Geometry uses the reference's formulas (MeshGmsh.cpp, Element.cpp,
// MeshCommon.cpp) in the same operation order, including its quirks:
//   Q1 cell "volume" = sum_f (face centre . S) = 3 x the true volume (MeshGmsh.cpp:101-133);
//   Q2 cell "centroid" = (v0 + v1 + 2 v2)/4 (MeshGmsh.cpp:135-145);
//   Q13 MUSCL face vector lookup through a face-id map keyed before ids exist
//       (Element.cpp:102-105, 185-187): slot 3 for face 0, slot 0 otherwise.
#include "mesh_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <numeric>
#include <thread>

namespace bes {

// colours of the block-ILU(0) schedule (balanced colouring of the renumbering)
constexpr int kBalancedColours = 5;

namespace {

const int kTetFace[4][3] = {{0, 2, 1}, {1, 2, 3}, {0, 3, 2}, {0, 1, 3}};

// Threads of the host mesh build: the BES_HOST_THREADS environment variable if set (>= 1),
// else the hardware's, at most 16.
int64_t host_threads() {
  static const int64_t n = [] {
    const char* e = std::getenv("BES_HOST_THREADS");
    const int64_t want = e ? std::atoll(e) : 0;
    const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
    return std::min<int64_t>(want >= 1 ? want : hw, 16);
  }();
  return n;
}

// body(begin, end) over [0, n) in contiguous chunks on up to host_threads() threads.  Every
// index is handled by exactly one call, so a loop whose iterations write disjoint elements and
// read only what earlier loops wrote gives the serial loop's result.  A chunk whose thread
// cannot be started runs on the calling thread.
template <class F>
void parallel_for(int64_t n, F&& body) {
  const int64_t kMinChunk = 1 << 15;
  const int64_t nt = std::min<int64_t>(host_threads(), (n + kMinChunk - 1) / kMinChunk);
  if (nt <= 1) {
    if (n > 0) body((int64_t)0, n);
    return;
  }
  const int64_t chunk = (n + nt - 1) / nt;
  std::vector<std::thread> threads;
  threads.reserve((size_t)nt);
  for (int64_t t = 1; t < nt; ++t) {
    const int64_t b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    try {
      threads.emplace_back([&body, b, e] { body(b, e); });
    } catch (...) {
      body(b, e);
    }
  }
  body((int64_t)0, std::min(n, chunk));
  for (auto& th : threads) th.join();
}

inline void cross_ref(const double* a, const double* b, const double* c, double* r) {
  // (c - b) x (a - b)  (MeshMath::crossProduct, src/MeshCommon.cpp:77-96)
  r[0] = (c[1] - b[1]) * (a[2] - b[2]) - (a[1] - b[1]) * (c[2] - b[2]);
  r[1] = (a[0] - b[0]) * (c[2] - b[2]) - (c[0] - b[0]) * (a[2] - b[2]);
  r[2] = (c[0] - b[0]) * (a[1] - b[1]) - (a[0] - b[0]) * (c[1] - b[1]);
}

// Open-addressing hash map from a sorted vertex triple to a face id.
class FaceTable {
 public:
  explicit FaceTable(size_t expected) {
    size_t cap = 16;
    while (cap < expected * 2) cap <<= 1;
    mask_ = cap - 1;
    keys_.assign(cap * 3, -1);
    vals_.assign(cap, -1);
  }
  // returns existing id or inserts `id` and returns -1
  int64_t find_or_insert(const int64_t* k, int64_t id) {
    size_t h = hash(k) & mask_;
    while (true) {
      int64_t* slot = &keys_[h * 3];
      if (slot[0] < 0) {
        slot[0] = k[0];
        slot[1] = k[1];
        slot[2] = k[2];
        vals_[h] = id;
        return -1;
      }
      if (slot[0] == k[0] && slot[1] == k[1] && slot[2] == k[2]) return vals_[h];
      h = (h + 1) & mask_;
    }
  }
  void overwrite(const int64_t* k, int64_t id) {
    size_t h = hash(k) & mask_;
    while (true) {
      int64_t* slot = &keys_[h * 3];
      if (slot[0] < 0 || (slot[0] == k[0] && slot[1] == k[1] && slot[2] == k[2])) {
        slot[0] = k[0];
        slot[1] = k[1];
        slot[2] = k[2];
        vals_[h] = id;
        return;
      }
      h = (h + 1) & mask_;
    }
  }

 private:
  static size_t hash(const int64_t* k) {
    uint64_t h = (uint64_t)k[0] * 0x9E3779B97F4A7C15ull;
    h ^= (uint64_t)k[1] + 0xC2B2AE3D27D4EB4Full + (h << 6) + (h >> 2);
    h ^= (uint64_t)k[2] * 0x165667B19E3779F9ull + (h << 6) + (h >> 2);
    h ^= h >> 29;
    return (size_t)h;
  }
  size_t mask_;
  std::vector<int64_t> keys_;
  std::vector<int64_t> vals_;
};

inline void sort3(int64_t* k) {
  if (k[0] > k[1]) std::swap(k[0], k[1]);
  if (k[1] > k[2]) std::swap(k[1], k[2]);
  if (k[0] > k[1]) std::swap(k[0], k[1]);
}

// Per-cell data that follows from the faces, for cells with `nfc` faces (slots nfc..3 empty):
// neighbours, inverse-distance weights (Element::computeAllFaceInverseDistanceWeightage,
// src/Element.cpp:120-139), projected lengths (TimeStepCalculatorLocal::computeProjectedLength_,
// src/TimeStepCalculatorLocal.cpp:51-63) and the MUSCL face-vector slot (Q13: the local face
// map is keyed by face id 0 for every face, so face 0 resolves to the cell's last slot).
void cell_links(RefMesh& M, int nfc, bool muscl_exact) {
  const int64_t nc = M.nc;
  parallel_for(nc, [&](int64_t c0, int64_t c1) {
  for (int64_t c = c0; c < c1; ++c) {
    for (int m = 0; m < nfc; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      if (M.kind[f] == KIND_INTERNAL) M.cadj[c * 4 + m] = (M.owner[f] != c) ? M.owner[f] : M.neigh[f];
    }
    for (int m = 0; m < nfc; ++m) {
      const int64_t a = M.cadj[c * 4 + m];
      if (a < 0) continue;
      const int64_t f = M.cface[c * 4 + m];
      double d1 = 0, d2 = 0;
      for (int d = 0; d < 3; ++d) {
        const double x1 = M.centroid[c * 3 + d] - M.center[f * 3 + d];
        const double x2 = M.centroid[a * 3 + d] - M.center[f * 3 + d];
        d1 += x1 * x1;
        d2 += x2 * x2;
      }
      d1 = std::sqrt(d1);
      d2 = std::sqrt(d2);
      M.weight[c * 4 + m] = d2 / (d1 + d2);
    }
    for (int m = 0; m < nfc; ++m)
      for (int d = 0; d < 3; ++d) M.plen[c * 3 + d] += std::fabs(M.S[M.cface[c * 4 + m] * 3 + d]);
    for (int d = 0; d < 3; ++d) M.plen[c * 3 + d] /= 2.0;
    for (int m = 0; m < nfc; ++m)
      M.muscl_slot[c * 4 + m] =
          (int8_t)(muscl_exact ? m : (M.cface[c * 4 + m] == 0 ? nfc - 1 : 0));
  }
  });
}

// Triangle meshes (Mesh::readGmsh, src/Mesh.cpp:235-426; MeshGmsh.cpp:22-42, 71-93): boundary
// lines first in file order with normal (y1 - y0, x0 - x1); a triangle's edges are
// (v0,v1), (v1,v2), (v2,v0), a new edge takes that order (normal out of the triangle that
// creates it), and a boundary line is flipped when it opposes the triangle's outward normal
// (y_b - y_a, x_a - x_b) (MeshMath::computeTwoDimOutwardNormal, src/MeshCommon.cpp:60-67).
// Area 0.5 |(x0 - x1)(y2 - y1) - (x2 - x1)(y0 - y1)|, centroid (v0 + v1 + v2)/3.  Only x and y
// are read; z of every centre and normal is 0, and face slot 3 of every cell stays empty.
bool build_ref_mesh_2d(const double* X, int64_t nv, const int64_t* blines, const int32_t* btags,
                       int64_t nb, const int64_t* tris, int64_t nc, bool muscl_exact, RefMesh& M,
                       std::string& err) {
  M.dim = 2;
  const int64_t nf_est = (3 * nc + nb) / 2 + 16;
  M.S.reserve(nf_est * 3);
  M.nhat.reserve(nf_est * 3);
  M.center.reserve(nf_est * 3);
  M.area.reserve(nf_est);
  M.owner.reserve(nf_est);
  M.neigh.reserve(nf_est);
  M.kind.reserve(nf_est);
  FaceTable table((size_t)nf_est);
  auto new_face = [&](int64_t v0, int64_t v1, int8_t kind) -> int64_t {
    const int64_t id = (int64_t)M.kind.size();
    const double* a = &X[v0 * 3];
    const double* b = &X[v1 * 3];
    const double S[2] = {b[1] - a[1], a[0] - b[0]};
    const double area = std::sqrt(S[0] * S[0] + S[1] * S[1]);
    for (int d = 0; d < 2; ++d) {
      M.S.push_back(S[d]);
      M.nhat.push_back(S[d] / area);
      M.center.push_back(0.5 * (a[d] + b[d]));
    }
    M.S.push_back(0.0);
    M.nhat.push_back(0.0);
    M.center.push_back(0.0);
    M.area.push_back(area);
    M.owner.push_back(-1);
    M.neigh.push_back(-1);
    M.kind.push_back(kind);
    return id;
  };
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t* v = &blines[b * 2];
    for (int q = 0; q < 2; ++q)
      if (v[q] < 0 || v[q] >= nv) {
        err = "boundary line references a missing node";
        return false;
      }
    int8_t kind;
    if (btags[b] == 1)
      kind = KIND_SLIP_WALL;
    else if (btags[b] == 2)
      kind = KIND_FREESTREAM;
    else {
      err = "boundary line with an unknown boundary tag " + std::to_string(btags[b]);
      return false;
    }
    int64_t k[3] = {std::min(v[0], v[1]), std::max(v[0], v[1]), -2};
    table.overwrite(k, new_face(v[0], v[1], kind));
  }
  M.nc = nc;
  M.cface.assign(nc * 4, -1);
  M.cadj.assign(nc * 4, -1);
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t* p = &tris[c * 3];
    for (int q = 0; q < 3; ++q)
      if (p[q] < 0 || p[q] >= nv) {
        err = "triangle references a missing node";
        return false;
      }
    for (int m = 0; m < 3; ++m) {
      const int64_t va = p[m], vb = p[(m + 1) % 3];
      int64_t k[3] = {std::min(va, vb), std::max(va, vb), -2};
      const int64_t next = (int64_t)M.kind.size();
      int64_t f = table.find_or_insert(k, next);
      if (f < 0) {
        f = new_face(va, vb, KIND_INTERNAL);
        M.owner[f] = c;
      } else if (M.kind[f] != KIND_INTERNAL) {
        const double out[2] = {X[vb * 3 + 1] - X[va * 3 + 1], -X[vb * 3] + X[va * 3]};
        const double dp = M.S[f * 3] * out[0] + M.S[f * 3 + 1] * out[1];
        if (dp < 0)
          for (int d = 0; d < 2; ++d) {
            M.S[f * 3 + d] = -M.S[f * 3 + d];
            M.nhat[f * 3 + d] = -M.nhat[f * 3 + d];
          }
        M.owner[f] = c;
        M.neigh[f] = -1;
      } else {
        if (M.neigh[f] >= 0) {
          err = "an edge is shared by more than two triangles";
          return false;
        }
        M.neigh[f] = c;
      }
      M.cface[c * 4 + m] = f;
    }
  }
  M.nf = (int64_t)M.kind.size();
  for (int64_t f = 0; f < M.nf; ++f) {
    if (M.owner[f] < 0) {
      err = "boundary line " + std::to_string(f) + " is not an edge of any triangle";
      return false;
    }
    if (M.kind[f] == KIND_INTERNAL && M.neigh[f] < 0) {
      err = "edge " + std::to_string(f) +
            " belongs to one triangle only and no boundary line covers it";
      return false;
    }
  }
  M.vol.assign(nc, 0);
  M.centroid.assign(nc * 3, 0);
  M.rvec.assign(nc * 12, 0);
  M.weight.assign(nc * 4, 0);
  M.plen.assign(nc * 3, 0);
  M.muscl_slot.assign(nc * 4, 0);
  parallel_for(nc, [&](int64_t c0, int64_t c1) {
  for (int64_t c = c0; c < c1; ++c) {
    const double* x0 = &X[tris[c * 3] * 3];
    const double* x1 = &X[tris[c * 3 + 1] * 3];
    const double* x2 = &X[tris[c * 3 + 2] * 3];
    M.vol[c] = 0.5 * std::fabs((x0[0] - x1[0]) * (x2[1] - x1[1]) - (x2[0] - x1[0]) * (x0[1] - x1[1]));
    for (int d = 0; d < 2; ++d) M.centroid[c * 3 + d] = (x0[d] + x1[d] + x2[d]) / 3;
    for (int m = 0; m < 3; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      for (int d = 0; d < 2; ++d)
        M.rvec[c * 12 + m * 3 + d] = M.center[f * 3 + d] - M.centroid[c * 3 + d];
    }
  }
  });
  cell_links(M, 3, muscl_exact);
  return true;
}

}  // namespace

bool build_ref_mesh(const double* X, int64_t nv, const int64_t* btris, const int32_t* btags,
                    int64_t nb, const int64_t* tets, int64_t nc, int dim, bool muscl_exact,
                    RefMesh& M, std::string& err) {
  M = RefMesh();
  if (nc <= 0 || nv <= 0) {
    err = "empty mesh";
    return false;
  }
  if (dim == 2) return build_ref_mesh_2d(X, nv, btris, btags, nb, tets, nc, muscl_exact, M, err);
  if (dim != 3) {
    err = "mesh dimension must be 2 or 3";
    return false;
  }
  const int64_t nf_est = (4 * nc + nb) / 2 + 16;
  M.S.reserve(nf_est * 3);
  M.nhat.reserve(nf_est * 3);
  M.center.reserve(nf_est * 3);
  M.area.reserve(nf_est);
  M.owner.reserve(nf_est);
  M.neigh.reserve(nf_est);
  M.kind.reserve(nf_est);
  FaceTable table((size_t)nf_est);
  auto new_face = [&](const int64_t* v, int8_t kind) -> int64_t {
    const int64_t id = (int64_t)M.kind.size();
    double S[3], c[3];
    for (int d = 0; d < 3; ++d) c[d] = (X[v[0] * 3 + d] + X[v[1] * 3 + d] + X[v[2] * 3 + d]) / 3;
    cross_ref(&X[v[0] * 3], &X[v[1] * 3], &X[v[2] * 3], S);
    double a = 0;
    for (int d = 0; d < 3; ++d) {
      S[d] /= 2.0;
      a += S[d] * S[d];
    }
    a = std::sqrt(a);
    for (int d = 0; d < 3; ++d) {
      M.S.push_back(S[d]);
      M.nhat.push_back(S[d] / a);
      M.center.push_back(c[d]);
    }
    M.area.push_back(a);
    M.owner.push_back(-1);
    M.neigh.push_back(-1);
    M.kind.push_back(kind);
    return id;
  };
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t* v = &btris[b * 3];
    for (int q = 0; q < 3; ++q)
      if (v[q] < 0 || v[q] >= nv) {
        err = "boundary triangle references a missing node";
        return false;
      }
    int8_t kind;
    if (btags[b] == 1)
      kind = KIND_SLIP_WALL;
    else if (btags[b] == 2)
      kind = KIND_FREESTREAM;
    else {
      err = "boundary triangle with an unknown boundary tag " + std::to_string(btags[b]);
      return false;
    }
    int64_t k[3] = {v[0], v[1], v[2]};
    sort3(k);
    table.overwrite(k, new_face(v, kind));
  }
  M.nc = nc;
  M.cface.assign(nc * 4, -1);
  M.cadj.assign(nc * 4, -1);
  for (int64_t c = 0; c < nc; ++c) {
    const int64_t* p = &tets[c * 4];
    for (int q = 0; q < 4; ++q)
      if (p[q] < 0 || p[q] >= nv) {
        err = "tetrahedron references a missing node";
        return false;
      }
    for (int m = 0; m < 4; ++m) {
      const int64_t v[3] = {p[kTetFace[m][0]], p[kTetFace[m][1]], p[kTetFace[m][2]]};
      int64_t k[3] = {v[0], v[1], v[2]};
      sort3(k);
      const int64_t next = (int64_t)M.kind.size();
      int64_t f = table.find_or_insert(k, next);
      if (f < 0) {
        f = new_face(v, KIND_INTERNAL);
        M.owner[f] = c;
      } else if (M.kind[f] != KIND_INTERNAL) {
        double out[3];
        cross_ref(&X[v[0] * 3], &X[v[1] * 3], &X[v[2] * 3], out);
        const double dp = M.S[f * 3] * out[0] + M.S[f * 3 + 1] * out[1] + M.S[f * 3 + 2] * out[2];
        if (dp < 0)
          for (int d = 0; d < 3; ++d) {
            M.S[f * 3 + d] = -M.S[f * 3 + d];
            M.nhat[f * 3 + d] = -M.nhat[f * 3 + d];
          }
        M.owner[f] = c;
        M.neigh[f] = -1;
      } else {
        if (M.neigh[f] >= 0) {
          err = "a face is shared by more than two tetrahedra";
          return false;
        }
        M.neigh[f] = c;
      }
      M.cface[c * 4 + m] = f;
    }
  }
  M.nf = (int64_t)M.kind.size();
  for (int64_t f = 0; f < M.nf; ++f) {
    if (M.owner[f] < 0) {
      err = "boundary triangle " + std::to_string(f) + " is not a face of any tetrahedron";
      return false;
    }
    if (M.kind[f] == KIND_INTERNAL && M.neigh[f] < 0) {
      err = "face " + std::to_string(f) +
            " belongs to one tetrahedron only and no boundary triangle covers it";
      return false;
    }
  }
  M.vol.assign(nc, 0);
  M.centroid.assign(nc * 3, 0);
  M.rvec.assign(nc * 12, 0);
  M.weight.assign(nc * 4, 0);
  M.plen.assign(nc * 3, 0);
  M.muscl_slot.assign(nc * 4, 0);
  parallel_for(nc, [&](int64_t c0, int64_t c1) {
  for (int64_t c = c0; c < c1; ++c) {
    const int64_t* p = &tets[c * 4];
    for (int d = 0; d < 3; ++d)
      M.centroid[c * 3 + d] =
          (X[p[0] * 3 + d] + X[p[1] * 3 + d] + X[p[2] * 3 + d] + X[p[2] * 3 + d]) / 4;
    double V = 0;
    for (int m = 0; m < 4; ++m) {
      double S[3], C[3];
      const double* a = &X[p[kTetFace[m][0]] * 3];
      const double* b = &X[p[kTetFace[m][1]] * 3];
      const double* e = &X[p[kTetFace[m][2]] * 3];
      cross_ref(a, b, e, S);
      double dotp = 0;
      for (int d = 0; d < 3; ++d) {
        S[d] /= 2.0;
        C[d] = ((0.0 + a[d]) + b[d]) + e[d];
        C[d] /= 3.0;
      }
      for (int d = 0; d < 3; ++d) dotp += C[d] * S[d];
      V += dotp;
    }
    M.vol[c] = V;
    for (int m = 0; m < 4; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      for (int d = 0; d < 3; ++d)
        M.rvec[c * 12 + m * 3 + d] = M.center[f * 3 + d] - M.centroid[c * 3 + d];
    }
  }
  });
  cell_links(M, 4, muscl_exact);
  return true;
}

namespace {

// Reverse Cuthill-McKee on the cell adjacency graph, one BFS per connected component, started
// from a pseudo-peripheral cell (repeated BFS to the farthest lowest-degree cell).
std::vector<int64_t> rcm_order(const RefMesh& M) {
  const int64_t nc = M.nc;
  std::vector<int> deg(nc, 0);
  for (int64_t c = 0; c < nc; ++c)
    for (int m = 0; m < 4; ++m) deg[c] += M.cadj[c * 4 + m] >= 0;
  std::vector<int64_t> order;
  order.reserve(nc);
  std::vector<int64_t> level(nc, -1);
  std::vector<char> done(nc, 0);
  std::vector<int64_t> queue;
  queue.reserve(nc);
  auto bfs_far = [&](int64_t s) -> int64_t {
    queue.clear();
    queue.push_back(s);
    level[s] = 0;
    size_t h = 0;
    int64_t far = s;
    while (h < queue.size()) {
      const int64_t c = queue[h++];
      if (level[c] > level[far] || (level[c] == level[far] && deg[c] < deg[far])) far = c;
      for (int m = 0; m < 4; ++m) {
        const int64_t a = M.cadj[c * 4 + m];
        if (a >= 0 && level[a] < 0) {
          level[a] = level[c] + 1;
          queue.push_back(a);
        }
      }
    }
    for (int64_t c : queue) level[c] = -1;
    return far;
  };
  for (int64_t s0 = 0; s0 < nc; ++s0) {
    if (done[s0]) continue;
    int64_t s = bfs_far(s0);
    s = bfs_far(s);
    // Cuthill-McKee BFS from s, neighbours by increasing degree
    const size_t first = order.size();
    order.push_back(s);
    done[s] = 1;
    size_t h = first;
    while (h < order.size()) {
      const int64_t c = order[h++];
      int64_t nb[4];
      int k = 0;
      for (int m = 0; m < 4; ++m) {
        const int64_t a = M.cadj[c * 4 + m];
        if (a >= 0 && !done[a]) nb[k++] = a;
      }
      std::sort(nb, nb + k, [&](int64_t x, int64_t y) {
        return deg[x] != deg[y] ? deg[x] < deg[y] : x < y;
      });
      for (int q = 0; q < k; ++q) {
        done[nb[q]] = 1;
        order.push_back(nb[q]);
      }
    }
    std::reverse(order.begin() + first, order.end());
  }
  return order;
}

}  // namespace

void build_soa(const RefMesh& M, double venkat_k, bool muscl_exact, bool renumber, SoaMesh& S) {
  S = SoaMesh();
  const int64_t nc = M.nc, nf = M.nf;
  S.nc = (int32_t)nc;
  S.nf = (int32_t)nf;
  // ---- cells
  S.cell_new2ref = renumber ? rcm_order(M) : std::vector<int64_t>();
  if (!renumber) {
    S.cell_new2ref.resize(nc);
    std::iota(S.cell_new2ref.begin(), S.cell_new2ref.end(), 0);
  } else {
    // Colour-major numbering: a balanced colouring in RCM order (each cell takes, among the
    // kBalancedColours colours its coloured neighbours do not use, the one used least so far),
    // then cells sorted by (colour, RCM position).  Every colour of the block-ILU(0) sweeps is
    // then one contiguous range (coalesced loads) of about the same size (no latency-bound
    // small stages), and each range keeps the RCM locality.  A tetrahedron has at most four
    // neighbours, so five colours always suffice.  Measured with the oracle on the 72,000-cell
    // bump channel (implicit, CFL ramp 10 -> 1000): the balanced order needs 31 % fewer GMRES
    // iterations than first-fit colouring, whose last two colours hold 5 % and 2 % of the cells.
    std::vector<int32_t> col(nc, -1);
    std::vector<int64_t> count(32, 0);
    for (int64_t p = 0; p < nc; ++p) {
      const int64_t c = S.cell_new2ref[p];
      uint32_t used = 0;
      for (int m = 0; m < 4; ++m) {
        const int64_t a = M.cadj[c * 4 + m];
        if (a >= 0 && col[a] >= 0) used |= 1u << col[a];
      }
      int k = -1;
      for (int q = 0; q < kBalancedColours; ++q)
        if (!(used & (1u << q)) && (k < 0 || count[q] < count[k])) k = q;
      if (k < 0) {  // not reached for tetrahedra; first free colour beyond the set otherwise
        k = kBalancedColours;
        while (used & (1u << k)) ++k;
      }
      col[c] = k;
      ++count[k];
    }
    // Inside a colour, cells are grouped by which local faces lead to an earlier colour (the
    // lower neighbours of the block-ILU(0) sweeps), RCM order within a group: the rows of a
    // warp then read the same block slots in each sweep (whole sectors, no divergence).  Cells
    // of one colour are not coupled, so their order changes neither the factors nor the sweeps.
    std::vector<uint8_t> lowmask(nc, 0);
    for (int64_t c = 0; c < nc; ++c)
      for (int m = 0; m < 4; ++m) {
        const int64_t a = M.cadj[c * 4 + m];
        if (a >= 0 && col[a] < col[c]) lowmask[c] |= (uint8_t)(1u << m);
      }
    std::vector<int64_t> rank_ref(nc);
    for (int64_t p = 0; p < nc; ++p) rank_ref[S.cell_new2ref[p]] = p;
    {
      // stable counting sort by (colour, lower-neighbour pattern), RCM order inside a group
      int32_t maxcol = 0;
      for (int64_t c = 0; c < nc; ++c) maxcol = std::max(maxcol, col[c]);
      std::vector<int64_t> start((size_t)(maxcol + 1) * 16 + 1, 0);
      for (int64_t c = 0; c < nc; ++c) ++start[(size_t)col[c] * 16 + lowmask[c] + 1];
      for (size_t k = 1; k < start.size(); ++k) start[k] += start[k - 1];
      std::vector<int64_t> sorted(nc);
      for (int64_t p = 0; p < nc; ++p) {
        const int64_t c = S.cell_new2ref[p];
        sorted[start[(size_t)col[c] * 16 + lowmask[c]]++] = c;
      }
      S.cell_new2ref.swap(sorted);
    }
    S.rcm_rank.resize(nc);
    for (int64_t i = 0; i < nc; ++i) S.rcm_rank[i] = rank_ref[S.cell_new2ref[i]];
    S.cell_color.resize(nc);
    for (int64_t i = 0; i < nc; ++i) S.cell_color[i] = col[S.cell_new2ref[i]];
  }
  if (S.rcm_rank.empty()) {
    S.rcm_rank.resize(nc);
    std::iota(S.rcm_rank.begin(), S.rcm_rank.end(), 0);
  }
  S.cell_ref2new.assign(nc, -1);
  for (int64_t i = 0; i < nc; ++i) S.cell_ref2new[S.cell_new2ref[i]] = i;
  // ---- faces: interior sorted by (new owner, new neighbour), then slip walls, then
  // freestream, each group by new owner
  std::vector<int64_t> fi, fs, ff;
  for (int64_t f = 0; f < nf; ++f) {
    if (M.kind[f] == KIND_INTERNAL)
      fi.push_back(f);
    else if (M.kind[f] == KIND_SLIP_WALL)
      fs.push_back(f);
    else
      ff.push_back(f);
  }
  // order by (new owner, new neighbour or -1, reference id): the keys are computed once, so
  // the sort compares integers instead of looking the renumbering up per comparison
  auto sort_by_owner = [&](std::vector<int64_t>& ids) {
    struct Key {
      int64_t owner, neigh, id;
    };
    std::vector<Key> keys(ids.size());
    parallel_for((int64_t)ids.size(), [&](int64_t q0, int64_t q1) {
      for (int64_t q = q0; q < q1; ++q) {
        const int64_t f = ids[q];
        keys[q] = {S.cell_ref2new[M.owner[f]], M.neigh[f] >= 0 ? S.cell_ref2new[M.neigh[f]] : -1, f};
      }
    });
    std::sort(keys.begin(), keys.end(), [](const Key& a, const Key& b) {
      if (a.owner != b.owner) return a.owner < b.owner;
      if (a.neigh != b.neigh) return a.neigh < b.neigh;
      return a.id < b.id;
    });
    for (size_t q = 0; q < ids.size(); ++q) ids[q] = keys[q].id;
  };
  sort_by_owner(fi);
  sort_by_owner(fs);
  sort_by_owner(ff);
  S.nf_int = (int32_t)fi.size();
  S.nf_slip = (int32_t)fs.size();
  S.nf_free = (int32_t)ff.size();
  S.face_new2ref.clear();
  S.face_new2ref.insert(S.face_new2ref.end(), fi.begin(), fi.end());
  S.face_new2ref.insert(S.face_new2ref.end(), fs.begin(), fs.end());
  S.face_new2ref.insert(S.face_new2ref.end(), ff.begin(), ff.end());
  S.face_ref2new.assign(nf, -1);
  for (int64_t i = 0; i < nf; ++i) S.face_ref2new[S.face_new2ref[i]] = i;

  // ---- reconstructed-state slots
  S.nslots = muscl_exact ? 4 : 1;
  // extra (cell, m) pairs whose reference lookup slot is not the cell's main slot 0
  std::vector<std::pair<int32_t, uint8_t>> extras;
  if (!muscl_exact)
    for (int64_t i = 0; i < nc; ++i) {
      const int64_t c = S.cell_new2ref[i];
      for (int m = 0; m < 4; ++m) {
        const int slot = M.muscl_slot[c * 4 + m];
        if (slot != 0) {
          bool seen = false;
          for (auto& e : extras)
            if (e.first == (int32_t)i && e.second == (uint8_t)slot) seen = true;
          if (!seen) extras.push_back({(int32_t)i, (uint8_t)slot});
        }
      }
    }
  std::sort(extras.begin(), extras.end());
  S.n_extra = (int32_t)extras.size();
  for (auto& e : extras) {
    S.extra_cell.push_back(e.first);
    S.extra_m.push_back(e.second);
  }
  auto rs_index = [&](int64_t cnew, int slot) -> int32_t {
    if (muscl_exact) return (int32_t)(slot * nc + cnew);
    if (slot == 0) return (int32_t)cnew;
    for (int32_t k = 0; k < S.n_extra; ++k)
      if (S.extra_cell[k] == cnew && S.extra_m[k] == slot) return (int32_t)(nc * S.nslots + k);
    return -1;
  };

  // ---- cell arrays
  S.vol.resize(nc);
  S.inv_vol.resize(nc);
  S.eps2.resize(nc);
  S.plen.resize(3 * nc);
  S.adj.resize(4 * nc);
  S.cface.resize(4 * nc);
  S.gface.resize(4 * nc);
  S.Sc.resize(12 * nc);
  S.w.resize(4 * nc);
  S.r.resize(12 * nc);
  S.cflags.assign(nc, 0);
  parallel_for(nc, [&](int64_t i0, int64_t i1) {
  for (int64_t i = i0; i < i1; ++i) {
    const int64_t c = S.cell_new2ref[i];
    S.vol[i] = M.vol[c];
    S.inv_vol[i] = 1.0 / M.vol[c];
    // epsilon of LimiterVenkatakrishnan (src/LimiterVenkatakrishnan.cpp:42-46), squared
    const double eps = std::pow(venkat_k * std::pow(M.vol[c], 1.0 / M.dim), 3.0 / 2.0);
    S.eps2[i] = eps * eps;
    for (int d = 0; d < 3; ++d) S.plen[d * nc + i] = M.plen[c * 3 + d];
    int order[4] = {0, 1, 2, 3};
    // faces in reference-id order, an empty slot last
    auto key = [&](int m) { return M.cface[c * 4 + m] < 0 ? INT64_MAX : M.cface[c * 4 + m]; };
    std::sort(order, order + 4, [&](int a, int b) { return key(a) < key(b); });
    for (int m = 0; m < 4; ++m) {
      const int64_t f = M.cface[c * 4 + m];
      const int64_t a = M.cadj[c * 4 + m];
      if (f < 0) {
        // empty slot of a triangle: no neighbour, no area, weight 0, no face
        S.adj[m * nc + i] = -1;
        S.cface[m * nc + i] = -1;
        for (int d = 0; d < 3; ++d) {
          S.Sc[(m * 3 + d) * nc + i] = 0.0;
          S.r[(m * 3 + d) * nc + i] = 0.0;
        }
        S.w[m * nc + i] = 0.0;
        continue;
      }
      S.adj[m * nc + i] = a >= 0 ? (int32_t)S.cell_ref2new[a] : -1;
      S.cface[m * nc + i] = (int32_t)S.face_ref2new[f];
      const double sgn = (M.owner[f] == c) ? 1.0 : -1.0;
      for (int d = 0; d < 3; ++d) {
        S.Sc[(m * 3 + d) * nc + i] = sgn * M.S[f * 3 + d];
        S.r[(m * 3 + d) * nc + i] = M.rvec[c * 12 + m * 3 + d];
      }
      S.w[m * nc + i] = M.weight[c * 4 + m];
      if (M.kind[f] == KIND_SLIP_WALL) S.cflags[i] |= (uint8_t)(1u << m);
    }
    for (int m = 0; m < 4; ++m) {
      const int64_t fo = M.cface[c * 4 + order[m]];
      if (fo < 0) {
        S.gface[m * nc + i] = kNoFace;
        continue;
      }
      const int32_t fnew = (int32_t)S.face_ref2new[fo];
      S.gface[m * nc + i] = (M.owner[fo] == c) ? fnew : ~fnew;
    }
  }
  });
  for (int32_t k = 0; k < S.n_extra; ++k) S.cflags[S.extra_cell[k]] |= 0x10;

  // ---- face arrays
  S.fown.resize(nf);
  S.fnb.resize(nf);
  S.fsrc_own.resize(nf);
  S.fsrc_nb.resize(nf);
  S.fn.resize(3 * nf);
  S.farea.resize(nf);
  parallel_for(nf, [&](int64_t j0, int64_t j1) {
  for (int64_t j = j0; j < j1; ++j) {
    const int64_t f = S.face_new2ref[j];
    const int64_t o = M.owner[f], n = M.neigh[f];
    const int64_t on = S.cell_ref2new[o];
    S.fown[j] = (int32_t)on;
    S.fnb[j] = n >= 0 ? (int32_t)S.cell_ref2new[n] : -1;
    int mo = -1, mn = -1;
    for (int m = 0; m < 4; ++m) {
      if (M.cface[o * 4 + m] == f) mo = m;
      if (n >= 0 && M.cface[n * 4 + m] == f) mn = m;
    }
    S.fsrc_own[j] = rs_index(on, M.muscl_slot[o * 4 + mo]);
    S.fsrc_nb[j] = n >= 0 ? rs_index(S.cell_ref2new[n], M.muscl_slot[n * 4 + mn]) : -1;
    for (int d = 0; d < 3; ++d) S.fn[d * nf + j] = M.nhat[f * 3 + d];
    S.farea[j] = M.area[f];
  }
  });

  // ---- ELL slots of each face in its two cells
  S.f_m_own.assign(nf, -1);
  S.f_m_nb.assign(nf, -1);
  parallel_for(nf, [&](int64_t j0, int64_t j1) {
    for (int64_t j = j0; j < j1; ++j) {
      const int32_t o = S.fown[j], n = S.fnb[j];
      for (int m = 0; m < 4; ++m) {
        if (S.cface[m * nc + o] == j) S.f_m_own[j] = (int8_t)m;
        if (n >= 0 && S.cface[m * nc + n] == j) S.f_m_nb[j] = (int8_t)m;
      }
    }
  });
  // ---- colouring of the cell graph (no two adjacent cells share a colour): the balanced
  // colouring of the renumbering, or first fit in the given order without renumbering
  int32_t ncol = 0;
  if (!renumber) {
    S.cell_color.assign(nc, -1);
    for (int64_t i = 0; i < nc; ++i) {
      uint32_t used = 0;
      for (int m = 0; m < 4; ++m) {
        const int32_t a = S.adj[m * nc + i];
        if (a >= 0 && S.cell_color[a] >= 0) used |= 1u << S.cell_color[a];
      }
      int col = 0;
      while (used & (1u << col)) ++col;
      S.cell_color[i] = col;
    }
  }
  for (int64_t i = 0; i < nc; ++i) ncol = std::max(ncol, S.cell_color[i] + 1);
  S.n_colors = ncol;
  build_ilu_schedule(S, false);
}

void build_ilu_schedule(SoaMesh& S, bool rcm_order) {
  const int64_t nc = S.nc;
  S.ilu_pos.assign(nc, 0);
  std::vector<int32_t> stage(nc, 0);
  int32_t nst = 0;
  if (!rcm_order) {
    // colour order: position = (colour, id); with colour-major numbering this is the identity
    std::vector<int64_t> idx(nc);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int64_t a, int64_t b) { return S.cell_color[a] < S.cell_color[b]; });
    for (int64_t p = 0; p < nc; ++p) S.ilu_pos[idx[p]] = (int32_t)p;
    for (int64_t i = 0; i < nc; ++i) stage[i] = S.cell_color[i];
    nst = S.n_colors;
  } else {
    // RCM order with level scheduling: level(i) = 1 + max level of its earlier neighbours
    std::vector<int64_t> idx(nc);
    for (int64_t i = 0; i < nc; ++i) idx[S.rcm_rank[i]] = i;
    for (int64_t p = 0; p < nc; ++p) S.ilu_pos[idx[p]] = (int32_t)p;
    for (int64_t p = 0; p < nc; ++p) {
      const int64_t i = idx[p];
      int32_t lv = 0;
      for (int m = 0; m < 4; ++m) {
        const int32_t a = S.adj[m * nc + i];
        if (a >= 0 && S.ilu_pos[a] < p) lv = std::max(lv, stage[a] + 1);
      }
      stage[i] = lv;
      nst = std::max(nst, lv + 1);
    }
  }
  S.n_stages = nst;
  S.stage_off.assign(nst + 1, 0);
  for (int64_t i = 0; i < nc; ++i) S.stage_off[stage[i] + 1]++;
  for (int k = 0; k < nst; ++k) S.stage_off[k + 1] += S.stage_off[k];
  S.stage_rows.assign(nc, 0);
  std::vector<int32_t> fill(S.stage_off.begin(), S.stage_off.end() - 1);
  for (int64_t i = 0; i < nc; ++i) S.stage_rows[fill[stage[i]]++] = (int32_t)i;
}

}  // namespace bes
