// Production kernels, fused multiply-add allowed: the FP64 path (all FP64)
// and the FP32 path (FP32 reconstruction and flux; state, residual sums and
// update as unevaluated FP32 pairs with compensated sums, no FP64
// instruction except the last stage's norm epilogue).
#include "devtypes.hpp"
#include "mesh.hpp"
#include "physics.cuh"

namespace mst {
namespace fast {
constexpr bool kExactArith = false;
#include "kernels.inc"
#include "implicit.inc"

cudaError_t launch_gradient(int prec, const DevMesh& m, const double4_32a* q,
                            void* grad, int quirks, cudaStream_t s) {
  if (prec == kPrecF32)
    return gradient_t<float>(m, q, nullptr, grad, quirks, 0.0, nullptr, nullptr, nullptr, s);
  return gradient_t<double>(m, q, nullptr, grad, quirks, 0.0, nullptr, nullptr, nullptr, s);
}
cudaError_t launch_gradient_dt(int prec, const DevMesh& m, const double4_32a* q,
                               const float4* qf, void* grad, int quirks, double cfl,
                               double* dt_cell, float2* dt_cell_ff, double* dt_part,
                               cudaStream_t s) {
  if (prec == kPrecF32)
    return gradient_t<float>(m, q, qf, grad, quirks, cfl, dt_cell, dt_cell_ff, dt_part, s);
  return gradient_t<double>(m, q, nullptr, grad, quirks, cfl, dt_cell, nullptr, dt_part, s);
}
cudaError_t launch_to_f32(const double4_32a* q, float4* qf, int n, cudaStream_t s) {
  k_to_f32<<<(n + 255) / 256, 256, 0, s>>>(q, qf, n);
  return cudaGetLastError();
}
cudaError_t launch_flux_update(int prec, int flux, int order, const DevMesh& m,
                               const StepArgs& a, int, cudaStream_t s) {
  if (prec == kPrecF32) return flux_dispatch<float>(flux, order, m, a, s);
  return flux_dispatch<double>(flux, order, m, a, s);
}
cudaError_t launch_face_flux(int prec, int flux, int order, const DevMesh& m,
                             const StepArgs& a, double* F, cudaStream_t s) {
  if (prec == kPrecF32) return face_dispatch<float>(flux, order, m, a, F, s);
  return face_dispatch<double>(flux, order, m, a, F, s);
}
cudaError_t launch_spectral_dt(int prec, const DevMesh& m, const double4_32a* q,
                               double cfl, double* dt_cell, double* partials,
                               cudaStream_t s) {
  const int nb = (m.n_cells + 255) / 256;
  if (prec == kPrecF32)
    k_spectral_dt<float><<<nb, 256, 0, s>>>(m, q, cfl, dt_cell, partials);
  else
    k_spectral_dt<double><<<nb, 256, 0, s>>>(m, q, cfl, dt_cell, partials);
  return cudaGetLastError();
}
}  // namespace fast
}  // namespace mst
