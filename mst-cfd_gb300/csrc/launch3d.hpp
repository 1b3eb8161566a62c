// Launchers of the 3D residual kernels, one set per arithmetic variant
// (kernels3d_exact.cu: FP64 without FMA; kernels3d_fast.cu: FP64 and FP32).
#pragma once
#include <cuda_runtime.h>

#include "devtypes3d.hpp"

namespace mst {
#define MST_LAUNCH3D_DECLS                                                                   \
  /* gradient of the stage state into grad; with dt_part also the CFL   \
     step's per-block minima */                                                              \
  cudaError_t gradient(int prec, const DevMesh3& m, const Step3Args& a, void* grad,         \
                       double cfl, double* dt_part, cudaStream_t s);                        \
  /* mode 0: FP64 update, 1: FP32 float-pair update, 3: residual only */                    \
  cudaError_t flux_update(int prec, int order, bool visc, int mode, const DevMesh3& m,      \
                          const Step3Args& a, cudaStream_t s);                              \
  cudaError_t finalize_dt(const double* part, int n, double t_end, double* scal,            \
                          float* dt_ff, cudaStream_t s);                                    \
  cudaError_t kinetic(int prec, const DevMesh3& m, const Step3Args& a, double* part,        \
                      double* out, cudaStream_t s);                                         \
  cudaError_t pairs(bool to_pairs, double* q, int n, float4* h4, float* h1, float4* l4,     \
                    float* l1, cudaStream_t s);
namespace exact3 {
MST_LAUNCH3D_DECLS
}
namespace fast3 {
MST_LAUNCH3D_DECLS
}
#undef MST_LAUNCH3D_DECLS
}  // namespace mst
