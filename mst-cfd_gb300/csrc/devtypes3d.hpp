// Device-side views of the 3D residual path (kernels3d.inc).
#pragma once
#include <cuda_runtime.h>

#include "smem_limit.hpp"

namespace mst {

// Gradient record per cell: [3][5] plus one pad, so that a cell's gradient
// is 64 B (FP32) or 128 B (FP64), loaded and stored as aligned vectors.
constexpr int kGrad3 = 16;

// 3D mesh in device order (mesh3d.hpp DevLayout3D): FP64 vectors of 3
// packed (x, y, z) per face or cell-face, and FP32 copies packed in float4
struct DevMesh3 {
  int n_cells, n_faces, n_tiles, max_tile_faces;
  const int2* f_c0c1;
  const int* f_info;
  const double *f_dir, *f_r0, *f_r1, *f_eta;
  // FP32 copies packed for one 16-byte load each: (S, eta0), (r0, 0), (r1, 0)
  const float4 *f_dir_eta32, *f_r0_32, *f_r1_32;
  const double* c_vol;
  const double* c_ivol;     // 1/V
  const float2* c_ivol_ff;  // 1/V as a float pair
  const int* c_ptr;
  const int* cf_slot;       // tile slot << 1 | (cell is c1 of the face)
  const int* cf_nb;         // neighbour device cell, -1 on boundary faces
  const double* cf_w;       // [tot][2] face-value weights (self, neighbour)
  const double* cf_dir;     // [tot][3] outward area vector
  // FP32 copies: (outward S, self weight) and the neighbour weight
  const float4* cf_dw32;
  const float* cf_w1_32;
  const int *t_own_ptr, *t_bor_ptr, *t_bor;
};

// One stage of the 3D path.  FP64 state: q [nC][5].  FP32 path: the state
// as float pairs, hi parts (h4 = rho, rho u, rho v, rho w; h1 = E) and lo
// parts (l4, l1).
struct Step3Args {
  const double* q;        // state the residual is evaluated on (FP64)
  double* qn;             // updated state (FP64)
  const double* q0;       // Q^n for the second RK stage (FP64)
  const float4* h4;
  const float* h1;
  const float4* l4;
  const float* l1;
  float4* nh4;
  float* nh1;
  float4* nl4;
  float* nl1;
  const float4* ph4;      // Q^n hi / lo for the second stage
  const float* ph1;
  const float4* pl4;
  const float* pl1;
  const void* grad;       // [nC][kGrad3] in the path's precision ([3][5] + pad)
  double* r_out;          // [nC][5] residual (residual-only launches)
  const double* scal;     // device [0] = dt (FP64 paths)
  const float* dt_ff;     // device dt as a float pair (FP32 path)
  int stage;              // 0: Q - dt/V R;  1: 0.5 Q0 + 0.5 (Q - dt/V R)
  int limiter;
  double mu, lam, kappa, cv;
  float mu_f, lam_f, kappa_f, cv_f;
  double inlet[5];
  float inlet_f[5];
};

}  // namespace mst
