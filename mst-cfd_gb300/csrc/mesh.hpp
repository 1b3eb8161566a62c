// Host-side mesh front end: Fluent .msh reader, reference-exact geometry and
// the device layout (locality renumbering, cell tiles, SoA/CSR arrays).
//
// Geometry follows the reference operation by operation (mesh/Face.cpp:8-19,
// mesh/Cell.cpp:6-50, mesh/MshBlock.cpp:238-334, :370-406); this file must be
// compiled with -ffp-contract=off so no multiply-add is fused on hosts whose
// compilers fuse by default (aarch64).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mst {

// Boundary kinds of the reference's face zones (RhoSolver.cpp:98-229).
enum ZoneType : int {
  kInterior = 2,
  kWall = 3,
  kOutlet = 5,
  kSymmetry = 7,
  kInlet = 10,
};

struct HostMesh {
  int n_nodes = 0, n_cells = 0, n_faces = 0, n_int_faces = 0;
  std::vector<int> zone;          // [nz][4] id, first (1-based), last, type
  std::vector<double> node_xy;    // [nN][2]
  std::vector<int> face_nodes;    // [nF][2]
  std::vector<int> face_cells;    // [nF][2], c1 = -1 on boundary
  std::vector<int> face_type;     // [nF]
  std::vector<double> c1_shift;   // [nF][2] periodic image shift (or empty)
  // geometry, file numbering
  std::vector<double> face_ctr, face_dir, face_area, face_eta0;
  std::vector<int> face_dac;
  std::vector<uint8_t> face_flag;       // reference flagLeftRight [nF][2]
  std::vector<uint8_t> face_flag_geo;   // geometric left/right [nF][2]
  std::vector<int> cell_ptr, cell_faces, cell_nb;
  std::vector<double> cell_dof, cell_eta0c, cell_ctr, cell_vol;
  std::vector<double> cell_face_ctr;    // [tot][2] face centre in cell frame
  std::vector<int> inner, bond1, bond2;
  // batches of independent cases (empty for one mesh): the case of every
  // face, and the first file cell of every case plus the end [n_cases+1]
  std::vector<int> face_case, case_cells;
  bool periodic() const { return !c1_shift.empty(); }
  int n_zones() const { return (int)zone.size() / 4; }
};

// A 3D mesh as MshBlock reads it with DIM 3 (mesh/MshBlock.cpp:436-789):
// triangular and quadrilateral faces (zones with a fixed node count, or
// mixed zones whose lines start with their node count), geometry by the
// reference's 3D formulas (Face.cpp:20-39, Cell.cpp:6-14 and :52-59), plus
// the corrected cell volume by the divergence theorem.
struct HostMesh3D {
  int n_nodes = 0, n_cells = 0, n_faces = 0, n_int_faces = 0;
  std::vector<int> zone;          // [nz][4] id, first, last, type
  std::vector<double> node_xyz;   // [nN][3]
  std::vector<int> face_ptr;      // [nF+1] into face_nodes
  std::vector<int> face_nodes;    // node ids of each face, in file order
  std::vector<int> face_cells;    // [nF][2], c1 = -1 on boundary
  std::vector<int> face_type;     // [nF]
  std::vector<double> face_ctr, face_dir, face_area, face_eta0, face_cmd;  // cmd: [nF][3]
  std::vector<int> face_dac;
  std::vector<uint8_t> face_flag;      // [nF][3] flagLeftRight where set
  std::vector<uint8_t> face_flag_set;  // [nF] 1 where the reference sets them
  std::vector<int> cell_ptr, cell_faces, cell_nb;
  std::vector<double> cell_dof, cell_eta0c, cell_ctr, cell_vol, cell_vol_fixed;
  std::vector<int> cell_node_ptr, cell_nodes;  // reader's node order
  std::vector<int> inner, bond1, bond2;
  std::vector<int> cell_nL;  // [nC] neighbours with a lower id (MshBlock.cpp:746-756)
};
int read_msh3d(const std::string& path, HostMesh3D* m, std::string* err);

// Status codes shared with the C ABI.
enum : int { kOk = 0, kEInval = 1, kEMesh = 2 };

int read_msh(const std::string& path, HostMesh* m, std::string* err);
int build_from_arrays(int n_nodes, const double* node_xy, int n_cells,
                      int n_faces, const int* face_nodes,
                      const int* face_cells, int n_zones, const int* zones,
                      const double* c1_shift, HostMesh* m, std::string* err);
// Geometry + derived connectivity; called by both builders.
int build_geometry(HostMesh* m, std::string* err);
// Disjoint union of independent meshes (a batch of cases): nodes, cells and
// faces of part k follow those of parts 0..k-1, with every id shifted; the
// geometry is copied, not recomputed; face_case / case_cells record the
// parts.  Only the corrected (quirk-free) face-value rule applies to a union.
int build_union(const std::vector<const HostMesh*>& parts, HostMesh* out,
                std::string* err);

// ---------------------------------------------------------------------------
// Device layout.  Cells are renumbered along a Morton curve of their
// centroids and cut into tiles of kTileCells consecutive device cells; each
// face is owned by the tile of its lower device cell, and a tile also lists
// the faces it borrows from other tiles (faces cut by the tile boundary).
// Within a cell the face order of the reference (ascending file face id) is
// kept, which is what makes the per-cell gather bit-identical.
// ---------------------------------------------------------------------------
constexpr int kTileCells = 128;

// face kinds packed into DevLayout::f_info
enum FaceKind : int {
  kKindInterior = 0,
  kKindInlet = 1,
  kKindWall = 2,
  kKindSymmetry = 3,
  kKindOutlet = 4,
  kKindNone = 5,  // zone types the reference does not handle: zero flux
};
// f_info bits: [0,3) kind, 3/4 reference flags (axis 0/1), 5/6 geometric flags
constexpr int kInfoFlagRef = 3;
constexpr int kInfoFlagGeo = 5;
constexpr int kInfoCaseShift = 8;  // batch case id of the face (bits 8..30)

// per-cell-face gradient record: cf_nb low 29 bits = neighbour device cell,
// top bits = face-value mode
enum : int { kFvInterp = 0, kFvSelf = 1, kFvNb = 2 };
constexpr int kFvShift = 29;

struct DevLayout {
  int n_cells = 0, n_faces = 0, n_tiles = 0, max_tile_faces = 0;
  std::vector<int> cell_perm;   // file cell -> device cell
  std::vector<int> cell_iperm;  // device cell -> file cell
  std::vector<int> face_perm;   // file face -> device face
  std::vector<int> face_iperm;  // device face -> file face
  // faces (device numbering)
  std::vector<int> f_c0c1;      // [nF][2] device cells (c1 = -1)
  std::vector<int> f_info;      // [nF]
  std::vector<double> f_dir;    // [nF][2]
  std::vector<double> f_r0;     // [nF][2]  x_f - x_c0
  std::vector<double> f_r1;     // [nF][2]  x_f - x_c1 (image); 0 on boundary
  // cells (device numbering)
  std::vector<double> c_vol;    // [nC]
  std::vector<int> c_ptr;       // [nC+1]
  std::vector<int> cf_face;     // [tot] device face id, ~id if dof = -dir
  std::vector<int> cf_slot;     // [tot] (tile-local face slot << 1) | neg
  std::vector<int> cf_nb;       // [tot] neighbour | (mode << kFvShift),
                                //       reference-quirk face values
  std::vector<int> cf_nb_fix;   // [tot] same with corrected boundary loops
  std::vector<double> cf_w;     // [tot][2] weights (self, neighbour)
  // tiles
  std::vector<int> t_own_ptr;   // [nT+1] owned face range (device ids)
  std::vector<int> t_bor_ptr;   // [nT+1] into t_bor
  std::vector<int> t_bor;       // borrowed device face ids
  // fused FP32 tile pass (gradients formed in shared memory): per tile a
  // table of its cells (local 0..kTileCells-1) followed by its halo cells
  // (outside the tile, sharing an interior face with a tile cell)
  std::vector<int> t_halo_ptr;  // [nT+1] into t_halo
  std::vector<int> t_halo;      // halo device cells, ascending per tile
  std::vector<int> t_slot_loc;  // per tile face slot (tile t's slots start at
                                // t_own_ptr[t] + t_bor_ptr[t]): local index
                                // of c0 | local index of c1 << 16 (0xFFFF:
                                // boundary face)
  std::vector<int> cf_nbl;      // [tot] local index of the neighbour in its
                                // cell's tile table | corrected face-value
                                // mode << 16
  int max_halo = 0;
  int n_halo_cells = 0;       // distinct cells in some tile's halo
  int n_halo_cell_faces = 0;  // their cell-faces
};

int build_layout(const HostMesh& m, bool renumber, DevLayout* L,
                 std::string* err);

}  // namespace mst
