// Host-side mesh pre-processing: the reference's face discovery and geometry, its quirks, and
// the GB300 renumbering into structure-of-arrays.
#pragma once
#include <climits>
#include <cstdint>
#include <string>
#include <vector>

namespace bes {

// gface entry of an empty face slot (slot 3 of a triangle); never a face id or its complement
constexpr int32_t kNoFace = INT32_MIN;

enum FaceKind : int8_t { KIND_INTERNAL = 0, KIND_SLIP_WALL = 1, KIND_FREESTREAM = 2 };

// Mesh with the reference's semantics, in reference numbering (src/Mesh.cpp:95-636).
struct RefMesh {
  int64_t nc = 0, nf = 0;
  int dim = 3;  // 2: triangles (face slot 3 of every cell is empty: cface = cadj = -1)
  std::vector<double> S, nhat, area, center;  // per face [3], [3], [1], [3]
  std::vector<int64_t> owner, neigh;          // neigh = -1 on boundary faces
  std::vector<int8_t> kind;
  std::vector<double> vol, centroid, rvec, weight, plen;  // [1], [3], [4][3], [4], [3] per cell
  std::vector<int64_t> cface, cadj;                       // [4] per cell
  std::vector<int8_t> muscl_slot;                         // [4] per cell
};

// Build from Gmsh-ordered arrays: dim 3 takes boundary triangles [nb][3] and tetrahedra
// [nc][4], dim 2 boundary lines [nb][2] and triangles [nc][3].  Returns false with a message
// on an unusable mesh.
bool build_ref_mesh(const double* X, int64_t nv, const int64_t* btris, const int32_t* btags,
                    int64_t nb, const int64_t* tets, int64_t nc, int dim, bool muscl_exact,
                    RefMesh& M, std::string& err);

// Device-ready arrays after renumbering (all vectors already in the device layout).
struct SoaMesh {
  int32_t nc = 0, nf = 0, nf_int = 0, nf_slip = 0, nf_free = 0;
  int32_t nslots = 1;   // reconstructed states per cell (1 reference lookup, 4 exact)
  int32_t n_extra = 0;  // extra reconstructed states (reference lookup hitting a slot != 0)
  std::vector<int64_t> cell_new2ref, cell_ref2new, face_new2ref, face_ref2new;
  // cells: SoA [k][nc]
  std::vector<double> vol, inv_vol, eps2, plen;  // plen [3][nc]
  std::vector<int32_t> adj, cface, gface;        // [4][nc]; gface: faces in reference-id order,
                                                 // ~f when the cell is the face's neighbour,
                                                 // kNoFace in empty slots (triangles)
  std::vector<double> Sc, w, r;                  // [4*3][nc], [4][nc], [4*3][nc]
  std::vector<uint8_t> cflags;                   // bit m: face m is a slip wall; bit 4: has extras
  std::vector<int32_t> extra_cell;               // [n_extra], sorted
  std::vector<uint8_t> extra_m;                  // [n_extra]
  // faces: SoA [k][nf]
  std::vector<int32_t> fown, fnb, fsrc_own, fsrc_nb;  // fnb = -1 on boundary faces
  std::vector<double> fn, farea;                      // [3][nf], [nf]
  // implicit matrix in ELL form: per cell, slot 0 = diagonal block, slot 1+m = the block of
  // the neighbour across local face m (empty for boundary faces).  This is the reference's
  // block pattern (CoefficientMatrix::initialize, src/CoefficientMatrix.cpp:114-164: the
  // diagonal block first, then neighbours in local face order) with fixed-width rows.
  std::vector<int8_t> f_m_own, f_m_nb;   // local face index of each face in owner / neighbour
  std::vector<int32_t> cell_color;       // greedy colouring of the cell graph
  int32_t n_colors = 0;
  // Block-ILU(0) schedule: the factorisation order (ilu_pos: cell -> position) and its
  // stages, groups of rows with no coupling to rows of the same or later stages, run one
  // stage at a time.  Colour order: one stage per colour.  RCM order: one stage per level
  // of the dependency graph (level scheduling).
  std::vector<int32_t> ilu_pos;          // cell -> position in the factorisation order
  std::vector<int32_t> stage_rows;       // cells grouped by stage
  std::vector<int32_t> stage_off;        // [n_stages+1] offsets into stage_rows
  int32_t n_stages = 0;
  std::vector<int64_t> rcm_rank;         // reverse Cuthill-McKee position of each new cell
};

// Reverse Cuthill-McKee renumbering + face grouping + SoA packing.
void build_soa(const RefMesh& M, double venkat_k, bool muscl_exact, bool renumber, SoaMesh& out);

// Block-ILU(0) schedule: rcm_order = false -> colour order (stage = colour), true -> reverse
// Cuthill-McKee order with level scheduling (stage = dependency level).
void build_ilu_schedule(SoaMesh& S, bool rcm_order);

}  // namespace bes
