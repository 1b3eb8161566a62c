// Device-resident mesh and per-launch arguments shared by the kernel
// translation units and the C ABI layer.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "smem_limit.hpp"

namespace mst {

// Mesh arrays in device numbering (see mesh.hpp DevLayout).  Geometry is
// held twice: FP64 for the exact and FP64 paths, FP32 for the FP32 path.
struct DevMesh {
  int n_cells, n_faces, n_tiles, max_tile_faces;
  const int2* f_c0c1;
  const int* f_info;
  const double2* f_dir;
  const double2* f_r0;
  const double2* f_r1;
  const float2* f_dir32;
  const float2* f_r0_32;
  const float2* f_r1_32;
  const double* f_eta;    // eta0 per face (viscous face interpolation)
  const float* f_eta32;
  const double* c_vol;
  const double* c_ivol;  // 1/V (production paths; the exact path divides)
  const float2* c_ivol_ff;  // 1/V as an unevaluated float pair (hi, lo)
  const int* c_ptr;
  const int* cf_face;
  const int* cf_slot;
  const int* cf_nb;
  const int* cf_nb_fix;
  const double2* cf_w;
  const float2* cf_w32;
  // area vector of every cell-face, pointing out of the cell (the signed
  // f_dir of cf_face): a contiguous load instead of a gather
  const double2* cf_dir;
  const float2* cf_dir32;
  const int* t_own_ptr;
  const int* t_bor_ptr;
  const int* t_bor;
  // fused FP32 tile pass (mesh.hpp DevLayout): halo cells per tile, local
  // cell indices of every tile face slot and of every cell-face neighbour
  const int* t_halo_ptr;
  const int* t_halo;
  const int* t_slot_loc;
  const int* cf_nbl;
  int max_halo;
  int deg3;  // every cell has three faces and c_ptr[c] = 3c (triangles)
  // batches (nullptr for a single mesh): the case of every device cell and
  // the iteration at which each case converged (-1 while it runs).  The
  // residual kernels skip the cells of converged cases: after the
  // iteration that converged them both state buffers hold the same state.
  const int* c_case;
  const int* case_conv;
  // batches in mixed precision: each case's residual phase (1: FP32, 0:
  // FP64) and the phase a launch evaluates; cells of cases in the other
  // phase are skipped like those of converged cases (nullptr: every case
  // in the launch's phase)
  const int* case_lo;
  int lo_want;
  // batches: the tiles the residual kernels visit (those holding cells of
  // unconverged cases) when most cases have converged; nullptr: all tiles
  const int* tile_list;
  int n_list;
};

// the cell-face range of device cell c: [3c, 3c + 3) without a load on
// meshes of triangles only
__device__ __forceinline__ int2 cell_face_range(const DevMesh& m, int c) {
  if (m.deg3) return make_int2(3 * c, 3 * c + 3);
  return make_int2(m.c_ptr[c], m.c_ptr[c + 1]);
}

// true when case k of a batch is in the other residual phase than the launch
__device__ __forceinline__ bool case_other_phase(const DevMesh& m, int k) {
  return m.case_lo && m.case_lo[k] != m.lo_want;
}
__device__ __forceinline__ bool cell_other_phase(const DevMesh& m, int c) {
  return m.case_lo && m.case_lo[m.c_case[c]] != m.lo_want;
}

// true when device cell c belongs to a converged case of a batch, or to a
// case in the other residual phase
__device__ __forceinline__ bool cell_case_done(const DevMesh& m, int c) {
  if (!m.case_conv) return false;
  const int k = m.c_case[c];
  return m.case_conv[k] >= 0 || case_other_phase(m, k);
}

// true when every cell of [c0, c1) belongs to a converged case or to one
// in the other residual phase (the cases are contiguous ranges of device
// cells)
__device__ __forceinline__ bool range_cases_done(const DevMesh& m, int c0, int c1) {
  if (!m.case_conv || c1 <= c0) return false;
  for (int k = m.c_case[c0], e = m.c_case[c1 - 1]; k <= e; ++k)
    if (m.case_conv[k] < 0 && !case_other_phase(m, k)) return false;
  return true;
}

// Number of doubles of per-tile partial norms: linf[4], l2[4], mass.
constexpr int kNormSlots = 9;

struct StepArgs {
  const double4_32a* q;   // state the residual is evaluated on
  const float4* qf;       // its FP32 copy (FP32 path; nullptr: convert q)
  float4* qfn;            // FP32 copy of the updated state (or nullptr)
  // FP32 path with the state as float pairs (value = hi + lo): qf/qfn are
  // the hi parts, these the lo parts; q0f/q0lo = Q^n for the second stage.
  // When qlo is nullptr the state is the FP64 q/q0/qn.
  const float4* qlo;
  float4* qlon;
  const float4* q0f;
  const float4* q0lo;
  float dt_ff[2];         // fixed step as a float pair (mst_solve)
  const float2* dt_cell_ff;  // local step per cell as float pairs (FP32 path)
  const float* dt_ff_dev; // step as a float pair on the device (or nullptr)
  const double4_32a* q0;  // Q^n for the second RK stage (else nullptr)
  double4_32a* qn;        // updated state
  const void* grad;       // [n_cells][2][4] in the path's precision
  double4_32a* r_out;     // optional per-cell residual
  const double* dt_dev;   // device scalar step (CFL modes) or nullptr
  const double* dt_cell;  // per-cell step (local CFL) or nullptr
  double dt;              // fixed step
  int stage;              // 0: Q - dt/V R;  1: 0.5 Q0 + 0.5 (Q - dt/V R)
  int quirks;             // reproduce the reference's quirks
  int tile_grad;          // FP32 pairs, 2nd order, corrected mode: the flux
                          // kernel forms the gradients itself (grad unused)
  int limiter;            // MST_LIMITER_*
  double inlet[4];
  int viscous;            // laminar viscous term on
  double mu, lam, kappa, cv;
  // the same constants rounded to FP32 once on the host, so FP32 kernels
  // convert nothing per face
  float inlet_f[4];
  float mu_f, lam_f, kappa_f, cv_f;
  // batches: per case kCaseWords numbers (inflow state[4], mu, lambda,
  // kappa, cv), indexed by the case id in the face's info word; nullptr
  // for a single case (the scalars above)
  const double* case_tab;
  const float* case_tab_f;
  // limiter freezing (residual-only launches of the implicit path): per
  // case 0 live, 1 record the ratios slope / (upwind difference) of every
  // limited face into phi [n_faces][2][4] (path precision), 2 use them
  const int* case_frozen;
  void* phi;
  double* partials;       // [n_tiles][kNormSlots] or nullptr
};
constexpr int kCaseWords = 8;

// Inflow state and viscous constants of a run into the step arguments.
inline void set_physics(StepArgs& a, const double inlet[4], int viscous, double mu,
                        double lam, double kappa, double cv) {
  for (int k = 0; k < 4; ++k) {
    a.inlet[k] = inlet[k];
    a.inlet_f[k] = (float)inlet[k];
  }
  a.viscous = viscous;
  a.mu = mu;
  a.lam = lam;
  a.kappa = kappa;
  a.cv = cv;
  a.mu_f = (float)mu;
  a.lam_f = (float)lam;
  a.kappa_f = (float)kappa;
  a.cv_f = (float)cv;
}

// Arguments of one LU-SGS sweep launch (implicit.inc).
struct LusgsArgs {
  const double4_32a* q;    // Q^n, device order
  const double4_32a* r;    // R(Q^n)
  double4_32a* dq;         // dQ* after the forward sweep, dQ after the backward
  double* diag;            // D_i (written by the forward sweep)
  double4_32a* qn;         // Q^{n+1} (backward sweep)
  float4* qfn;             // its FP32 copy, or nullptr
  const int* color;        // colour of every device cell
  const int* cells;        // the cells of the colour being swept
  int n;                   // their number
  int col;                 // the colour
  const int* c_case;       // case of every device cell (nullptr: case 0)
  const double* cfl;       // CFL number of every case
  const double* case_tab;  // per-case coefficients (mu at [4]) or nullptr
  double mu;               // viscosity of a single case
  int viscous;
  double omega;
  const int* conv_iter;    // [n_cases] converged cases keep their state
  const int* iter;         // iteration counter (already advanced by the norms)
  // FP32 sweeps (dqf != nullptr): FP32 state copy, dQ* / dQ in FP32, the
  // per-case coefficients in FP32
  const float4* qf;
  float4* dqf;
  const float* case_tab_f;
  float mu_f;
  double p_floor;          // temperature floor p >= p_floor * rho (0: off)
  int* case_bad;           // [n_cases] set to 1 when a swept state has a
                           // non-positive (or NaN) density or pressure
};

// Per-case residual norms and the CFL of the next iteration, one block per
// case over its contiguous device cells: L2 = sqrt(mean (R_rho / V)^2)
// (fixed-order block reduction: deterministic).  The first iteration's L2
// is kept; CFL = clamp(cfl0 * L2_first / L2, cfl0, cfl_max) (switched
// evolution relaxation); a case converges at the first iteration whose
// L2 / L2_first < tol.
struct CaseNormArgs {
  const double4_32a* r;
  const int* case_first;   // [n_cases + 1] device cell ranges
  double* first;           // [n_cases] L2 of iteration 0
  double* last;            // [n_cases] latest L2
  double* cfl;             // [n_cases]
  int* conv_iter;          // [n_cases] -1 until the case is done (converged
                           // or diverged): the iteration it finished at
  int* n_conv;             // number of finished cases
  int* diverged;           // [n_cases] 1 once the case's L2 is not finite
  int* iter;               // iteration counter (advanced by k_iter_advance)
  int* frozen;             // [n_cases] limiter-freezing state (or nullptr)
  double* l2_win;          // [n_cases] L2 at the last freezing-window check
  double* own_first;       // [n_cases] L2 of this run's first iteration (the
                           // freezing reference, whatever first[] holds)
  double* frz_best;        // [n_cases] best L2 since the limiter froze
  int* frz_best_it;        // [n_cases] and its iteration
  int refreeze_window;     // see mst_implicit_params (0: off)
  double cfl0, cfl_max, tol, freeze_tol;
  int first_fixed;         // first[] holds reference L2s set by the caller
  double* part;            // [n_cases][8] partial sums of (R_rho / V)^2
  const int* case_lo;      // [n_cases] 1 while a case's residual is FP32 (the
                           // freezing state machine waits for FP64), or nullptr
  const int* restart_it;   // [n_cases] iteration of the case's (re)start
  double* stall_best;      // [n_cases] best L2 of the stall test
  int* stall_best_it;      // [n_cases] and its iteration
  int stall_window;        // see mst_implicit_params (0: off)
};

// Precisions / schemes (mirrors of the public enums)
enum { kPrecExact = 0, kPrecF64 = 1, kPrecF32 = 2 };
enum { kFluxAusm = 0, kFluxRoe = 1 };

// Launchers implemented once per arithmetic translation unit.
#define MST_DECLARE_LAUNCHERS(NS)                                             \
  namespace NS {                                                              \
  cudaError_t launch_gradient(int prec, const DevMesh& m,                     \
                              const double4_32a* q, void* grad, int quirks,   \
                              cudaStream_t s);                                \
  cudaError_t launch_gradient_dt(int prec, const DevMesh& m,                  \
                                 const double4_32a* q, const float4* qf,      \
                                 void* grad, int quirks, double cfl,          \
                                 double* dt_cell, float2* dt_cell_ff,         \
                                 double* dt_part, cudaStream_t s);            \
  cudaError_t launch_to_f32(const double4_32a* q, float4* qf, int n,         \
                            cudaStream_t s);                                  \
  cudaError_t launch_flux_update(int prec, int flux, int order,              \
                                 const DevMesh& m, const StepArgs& a,         \
                                 int threads, cudaStream_t s);                \
  cudaError_t launch_face_flux(int prec, int flux, int order,                \
                               const DevMesh& m, const StepArgs& a,           \
                               double* F, cudaStream_t s);                    \
  cudaError_t launch_spectral_dt(int prec, const DevMesh& m,                 \
                                 const double4_32a* q, double cfl,            \
                                 double* dt_cell, double* partials,           \
                                 cudaStream_t s);                             \
  cudaError_t lusgs_forward_t(const DevMesh& m, const LusgsArgs& a,          \
                              int threads, cudaStream_t s);                   \
  cudaError_t lusgs_backward_t(const DevMesh& m, const LusgsArgs& a,         \
                               int threads, cudaStream_t s);                  \
  cudaError_t launch_cfl_dt_pairs(const DevMesh& m, const float4* qf,        \
                                  double cfl, float2* dt_cell_ff,             \
                                  double* dt_part, cudaStream_t s);           \
  cudaError_t case_norms_t(const DevMesh& m, const CaseNormArgs& a,          \
                           int n_cases, cudaStream_t s);                      \
  }

MST_DECLARE_LAUNCHERS(exact)
MST_DECLARE_LAUNCHERS(fast)

}  // namespace mst
