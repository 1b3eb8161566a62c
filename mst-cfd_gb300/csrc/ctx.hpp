// Internal definitions of the C ABI's opaque handles, shared by the
// translation units that implement entry points (capi.cu, noalloc.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/mstcfd.h"
#include "devtypes.hpp"
#include "mesh.hpp"

// Records msg as this thread's mst_last_error() text and returns s.
mst_status mst_internal_fail(mst_status s, const std::string& msg);

struct mst_mesh {
  mst::HostMesh host;
  mst::DevLayout lay;
};

struct mst_mesh3d {
  mst::HostMesh3D host;
  // meshes from arrays: x(c0 frame) - x(c1 frame) per face ([nF][3]) or
  // empty; from_arrays is true when the reference geometry was not built
  std::vector<double> c1_shift;
  bool from_arrays = false;
};

struct DevArrays {
  int2* f_c0c1 = nullptr;
  int* f_info = nullptr;
  double2 *f_dir = nullptr, *f_r0 = nullptr, *f_r1 = nullptr, *cf_w = nullptr,
          *cf_dir = nullptr;
  float2 *f_dir32 = nullptr, *f_r0_32 = nullptr, *f_r1_32 = nullptr, *cf_w32 = nullptr,
         *cf_dir32 = nullptr;
  double* f_eta = nullptr;
  float* f_eta32 = nullptr;
  double* c_vol = nullptr;
  double* c_ivol = nullptr;
  float2* c_ivol_ff = nullptr;
  int *c_ptr = nullptr, *cf_face = nullptr, *cf_slot = nullptr, *cf_nb = nullptr,
      *cf_nb_fix = nullptr, *t_own_ptr = nullptr, *t_bor_ptr = nullptr,
      *t_bor = nullptr, *cell_iperm = nullptr, *cell_perm = nullptr,
      *t_halo_ptr = nullptr, *t_halo = nullptr, *t_slot_loc = nullptr, *cf_nbl = nullptr;
};

struct mst_node_avg;  // result writer buffers (io.cu)
void mst_io_release(struct mst_ctx* c);

struct mst_ctx {
  const mst_mesh* mesh = nullptr;
  mst_params p{};
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  DevArrays d;
  mst::DevMesh dm{};
  double4_32a *q_old = nullptr, *q_new = nullptr, *q_stage = nullptr,
              *r = nullptr, *stage_in = nullptr;
  // FP32 path: state as float pairs, hi parts (qf_*) and lo parts (ql_*)
  float4 *qf_old = nullptr, *qf_new = nullptr, *qf_stage = nullptr;
  float4 *ql_old = nullptr, *ql_new = nullptr, *ql_stage = nullptr;
  void* grad = nullptr;
  double* flux = nullptr;      // [nF][8] debug output
  double* partials = nullptr;  // [max(nT, nBlocks)][kNormSlots]
  double* dt_part = nullptr;   // [nBlocks]
  double* dt_cell = nullptr;   // [nC]
  float2* dt_cell_ff = nullptr;  // [nC] local steps as float pairs (FP32 path)
  double* scal = nullptr;      // [0] dt, [1] time
  double* norms = nullptr;     // [kNormSlots + 2]
  int last_launches = 0;
  // per-kernel event timing
  bool profiling = false;
  struct Pending { int kernel; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::string> kname;
  std::vector<int> klaunch;
  std::vector<double> kms;
  bool timed = false;
  bool grad_valid = false;
  // every cell volume finite and positive: only then does a non-finite
  // residual mean divergence (the reference's own geometry gives NaN
  // volumes on degenerate quads, and its results carry them)
  bool volumes_ok = true;
  std::vector<void*> allocs;
  mst_node_avg* node_avg = nullptr;
  // host-buffer pipeline (mst_step_host_jobs): copy-in and copy-out
  // streams, two staging slots each way, and the norms of every job
  struct HostPipe {
    cudaStream_t in = nullptr, out = nullptr;
    double4_32a* slot_in[2] = {nullptr, nullptr};
    double4_32a* slot_out[2] = {nullptr, nullptr};
    cudaEvent_t in_ready[2] = {}, in_free[2] = {}, out_ready[2] = {}, out_free[2] = {};
    double* job_norms = nullptr;  // [cap][kNormSlots + 2], device
    int cap = 0;
  } pipe;
};

