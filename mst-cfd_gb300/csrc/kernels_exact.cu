// FP64 parity kernels: compiled with --fmad=false so every product and sum
// rounds separately, in the reference's order (bit-identical residuals).
#include "devtypes.hpp"
#include "mesh.hpp"
#include "physics.cuh"

namespace mst {
namespace exact {
constexpr bool kExactArith = true;
#include "kernels.inc"
#include "implicit.inc"

cudaError_t launch_gradient(int, const DevMesh& m, const double4_32a* q,
                            void* grad, int quirks, cudaStream_t s) {
  return gradient_t<double>(m, q, nullptr, grad, quirks, 0.0, nullptr, nullptr, nullptr, s);
}
cudaError_t launch_gradient_dt(int, const DevMesh& m, const double4_32a* q,
                               const float4*, void* grad, int quirks, double cfl,
                               double* dt_cell, float2*, double* dt_part, cudaStream_t s) {
  return gradient_t<double>(m, q, nullptr, grad, quirks, cfl, dt_cell, nullptr, dt_part, s);
}
cudaError_t launch_to_f32(const double4_32a* q, float4* qf, int n, cudaStream_t s) {
  k_to_f32<<<(n + 255) / 256, 256, 0, s>>>(q, qf, n);
  return cudaGetLastError();
}
cudaError_t launch_flux_update(int, int flux, int order, const DevMesh& m,
                               const StepArgs& a, int, cudaStream_t s) {
  return flux_dispatch<double>(flux, order, m, a, s);
}
cudaError_t launch_face_flux(int, int flux, int order, const DevMesh& m,
                             const StepArgs& a, double* F, cudaStream_t s) {
  return face_dispatch<double>(flux, order, m, a, F, s);
}
cudaError_t launch_spectral_dt(int, const DevMesh& m, const double4_32a* q,
                               double cfl, double* dt_cell, double* partials,
                               cudaStream_t s) {
  const int nb = (m.n_cells + 255) / 256;
  k_spectral_dt<double><<<nb, 256, 0, s>>>(m, q, cfl, dt_cell, partials);
  return cudaGetLastError();
}
}  // namespace exact
}  // namespace mst
