// 3D solver mesh: the corrected geometry of the 3D residual path and its
// device layout.
//
// The reference's own 3D geometry (read_msh3d) is kept as the reference
// computes it; the residual path uses corrected geometry instead, because
// the reference's 3D cell volume and quadrilateral area are wrong
// (mesh/Cell.cpp:52-59, mesh/Face.cpp:30-36):
//   face centre   mean of its nodes (Face.cpp:8-15)
//   area vector   1/2 (n1-n0) x (n2-n0) (triangle), 1/2 (n2-n0) x (n3-n1)
//                 (quadrilateral: exact for any four nodes), oriented out
//                 of c0
//   cell centre   mean of its face centres (Cell.cpp:6-14), in the cell's
//                 own frame (periodic faces carry the shift of c1's frame)
//   volume        divergence theorem, V = 1/3 sum (x_f - x_c) . S_out
//   eta0          |x_f - x_c1| / (|x_f - x_c0| + |x_f - x_c1|) (Face.cpp:62-69)
// Compiled with -ffp-contract=off: the operation order is the one of the
// checker's restatement, so both produce the same bits.
#pragma once
#include <string>
#include <vector>

#include "mesh.hpp"

namespace mst {

struct SolverMesh3D {
  int n_cells = 0, n_faces = 0;
  std::vector<int> face_cells, face_kind;       // kind: FaceKind
  std::vector<double> face_ctr, face_dir;       // [nF][3]; dir out of c0
  std::vector<double> r0, r1;                   // [nF][3] x_f - x_c0, x_f - x_c1
  std::vector<double> eta;                      // [nF], 1 on boundary faces
  std::vector<double> cell_ctr, cell_vol;       // [nC][3], [nC]
  std::vector<int> cell_ptr, cell_faces, cell_nb;  // faces ascending, nb = -1 on boundary
  std::vector<double> cell_dir, cell_w;         // [tot][3] outward, [tot][2] (self, nb)
};

// c1_shift: [nF][3] x(c0 frame) - x(c1 frame) of periodic faces, or empty
int build_solver3d(const HostMesh3D& h, const std::vector<double>& c1_shift,
                   SolverMesh3D* s, std::string* err);

// f_info bits of the 3D layout: [0,3) kind, 3..5 axis flags (c0 is the left
// state along axis d when its outward area vector has S_d >= 0)
constexpr int kInfo3Flag = 3;

struct DevLayout3D {
  int n_cells = 0, n_faces = 0, n_tiles = 0, max_tile_faces = 0;
  std::vector<int> cell_perm, cell_iperm;   // file <-> device cells
  std::vector<int> face_perm;               // file face -> device face
  std::vector<int> f_c0c1, f_info;          // [nF][2], [nF]
  std::vector<double> f_dir, f_r0, f_r1;    // [nF][3]
  std::vector<double> f_eta;                // [nF]
  std::vector<double> c_vol;                // [nC]
  std::vector<int> c_ptr, cf_slot, cf_nb;   // cf_slot = tile slot << 1 | (cell is c1)
  std::vector<double> cf_w, cf_dir;         // [tot][2], [tot][3]
  std::vector<int> t_own_ptr, t_bor_ptr, t_bor;
};

// Morton renumbering of the cell centres, tiles of kTileCells cells, faces
// owned by the tile of their lower device cell (as the 2D layout)
int build_layout3d(const SolverMesh3D& s, DevLayout3D* L, std::string* err);

}  // namespace mst
