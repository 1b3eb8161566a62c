// 3D production kernels: FP64 with fused multiply-add, and the FP32 path
// (FP32 reconstruction and flux, float-pair state and residual sums).
#include "devtypes3d.hpp"
#include "launch3d.hpp"
#include "mesh.hpp"
#include "physics.cuh"

namespace mst {
namespace fast3 {
constexpr bool kExactArith = false;
#include "kernels3d.inc"

cudaError_t gradient(int prec, const DevMesh3& m, const Step3Args& a, void* grad, double cfl,
                     double* dt_part, cudaStream_t s) {
  if (prec == 2) return gradient3_t<float, 1>(m, a, grad, cfl, dt_part, s);
  return gradient3_t<double, 0>(m, a, grad, cfl, dt_part, s);
}
cudaError_t flux_update(int prec, int order, bool visc, int mode, const DevMesh3& m,
                        const Step3Args& a, cudaStream_t s) {
  if (prec == 2) {
    if (mode == 3) return flux3_dispatch<float, 3>(order, visc, m, a, s);
    return flux3_dispatch<float, 1>(order, visc, m, a, s);
  }
  if (mode == 3) return flux3_dispatch<double, 3>(order, visc, m, a, s);
  return flux3_dispatch<double, 0>(order, visc, m, a, s);
}
cudaError_t finalize_dt(const double* part, int n, double t_end, double* scal, float* dt_ff,
                        cudaStream_t s) {
  return finalize_dt3(part, n, t_end, scal, dt_ff, s);
}
cudaError_t kinetic(int prec, const DevMesh3& m, const Step3Args& a, double* part, double* out,
                    cudaStream_t s) {
  if (prec == 2) return kinetic3_t<1>(m, a, part, out, s);
  return kinetic3_t<0>(m, a, part, out, s);
}
cudaError_t pairs(bool to_pairs, double* q, int n, float4* h4, float* h1, float4* l4, float* l1,
                  cudaStream_t s) {
  return pairs3(to_pairs, q, n, h4, h1, l4, l1, s);
}
}  // namespace fast3
}  // namespace mst
