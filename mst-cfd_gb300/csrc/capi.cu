// C ABI of the GB300 density-based residual path (include/mstcfd.h).
// No exception crosses the boundary; every CUDA error becomes MST_ECUDA with
// its text in mst_last_error().
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/mstcfd.h"
#include "ctx.hpp"
#include "devtypes.hpp"
#include "mesh.hpp"

using mst::kNormSlots;

namespace {

thread_local std::string g_err;

void release_pipe(mst_ctx* c);  // the host-buffer pipeline's streams and slots

mst_status fail(mst_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

#define CU(call)                                                          \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess)                                                \
      return fail(MST_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
cudaError_t upload(T** dst, const std::vector<T>& src) {
  *dst = nullptr;
  size_t n = std::max<size_t>(src.size(), 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void**)dst, n);
  if (e != cudaSuccess) return e;
  if (!src.empty()) e = cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

// ---- small orchestration kernels (not on the arithmetic-parity path) ----
// device state -> file order and back
__global__ void k_gather_rows(const double4_32a* __restrict__ src,
                              const int* __restrict__ idx,
                              double4_32a* __restrict__ dst, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}

// double state <-> float pairs (hi = (float)q, lo = (float)(q - hi)); both
// in device order
__global__ void k_to_pairs(const double4_32a* __restrict__ q, float4* __restrict__ hi,
                           float4* __restrict__ lo, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a v = q[i];
  const float4 h = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
  hi[i] = h;
  lo[i] = make_float4((float)(v.x - (double)h.x), (float)(v.y - (double)h.y),
                      (float)(v.z - (double)h.z), (float)(v.w - (double)h.w));
}
__global__ void k_to_pairs1(const double* __restrict__ v, float2* __restrict__ out, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float h = (float)v[i];
  out[i] = make_float2(h, (float)(v[i] - (double)h));
}

// pairs -> double, gathered through idx (idx = nullptr: same order)
__global__ void k_from_pairs(const float4* __restrict__ hi, const float4* __restrict__ lo,
                             const int* __restrict__ idx, double4_32a* __restrict__ q, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = idx ? idx[i] : i;
  const float4 h = hi[s], l = lo[s];
  q[i] = make_double4_32a((double)h.x + (double)l.x, (double)h.y + (double)l.y,
                          (double)h.z + (double)l.z, (double)h.w + (double)l.w);
}

// step length: fixed (mode 0) or min over block partials (mode 1), clipped
// so that the time reaches t_end; writes scal[0] = dt
__global__ void k_finalize_dt(const double* __restrict__ part, int n,
                              int mode, double dt_fixed, double t_end,
                              double* __restrict__ scal) {
  __shared__ double red[32];
  double x = 1e300;
  if (mode == 0) {
    x = dt_fixed;
  } else {
    for (int i = threadIdx.x; i < n; i += blockDim.x) x = (part[i] < x) ? part[i] : x;
    for (int o = 16; o > 0; o >>= 1) {
      double w = __shfl_xor_sync(0xffffffffu, x, o);
      x = (w < x) ? w : x;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      x = red[0];
      for (int i = 1; i < (int)(blockDim.x >> 5); ++i) x = (red[i] < x) ? red[i] : x;
    }
  }
  if (threadIdx.x == 0) {
    double t = scal[1];
    if (t_end > 0 && t + x > t_end) x = t_end - t;
    if (x < 0) x = 0;
    scal[0] = x;
    scal[1] = t + x;  // the step is always taken with this length
    // the same step as a float pair for the FP32 path (scal[2] as 2 floats)
    float* ff = reinterpret_cast<float*>(scal + 2);
    ff[0] = (float)x;
    ff[1] = (float)(x - (double)ff[0]);
  }
}

// norms of a step from per-tile partials (fixed order: deterministic).
// out: linf[4], l2[4] (sqrt(mean)), mass, dt, time
__global__ void k_finalize_norms(const double* __restrict__ part, int n_tiles,
                                 int n_cells, int advance,
                                 double* __restrict__ scal,
                                 double* __restrict__ out) {
  __shared__ double red[kNormSlots][32];
  const int j = threadIdx.y;  // one row of threads per norm slot
  double x = 0.0;
  for (int i = threadIdx.x; i < n_tiles; i += blockDim.x) {
    double v = part[(size_t)i * kNormSlots + j];
    x = (j < 4) ? ((x < v) ? v : x) : x + v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_xor_sync(0xffffffffu, x, o);
    x = (j < 4) ? ((x < w) ? w : x) : x + w;
  }
  if ((threadIdx.x & 31) == 0) red[j][threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = red[j][0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i)
      acc = (j < 4) ? ((acc < red[j][i]) ? red[j][i] : acc) : acc + red[j][i];
    if (j >= 4 && j < 8) acc = sqrt(acc / (double)n_cells);
    out[j] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0 && j == 0) {
    (void)advance;
    out[kNormSlots] = scal[0];
    out[kNormSlots + 1] = scal[1];
  }
}

}  // namespace

namespace {

int prec_of(const mst_params& p) { return p.precision; }

mst_status check_params(const mst_params* p) {
  if (!p) return fail(MST_EINVAL, "params is NULL");
  if (p->flux != MST_FLUX_AUSM && p->flux != MST_FLUX_ROE)
    return fail(MST_EINVAL, "unknown flux scheme");
  if (p->order != 1 && p->order != 2) return fail(MST_EINVAL, "order must be 1 or 2");
  if (p->limiter < MST_LIMITER_NONE || p->limiter > MST_LIMITER_VANALBADA)
    return fail(MST_EINVAL, "unknown limiter");
  if (p->precision < MST_PREC_FP64_EXACT || p->precision > MST_PREC_FP32)
    return fail(MST_EINVAL, "unknown precision");
  if (p->time_scheme != MST_TIME_EULER && p->time_scheme != MST_TIME_RK2)
    return fail(MST_EINVAL, "unknown time scheme");
  if (p->dt_mode < MST_DT_FIXED || p->dt_mode > MST_DT_CFL_LOCAL)
    return fail(MST_EINVAL, "unknown dt mode");
  if (p->dt_mode == MST_DT_FIXED && !(p->dt >= 0))
    return fail(MST_EINVAL, "dt must be >= 0");
  if (p->dt_mode != MST_DT_FIXED && !(p->cfl > 0))
    return fail(MST_EINVAL, "cfl must be > 0");
  if (p->viscous && p->order != 2)
    return fail(MST_EINVAL, "the viscous term needs order 2 (cell gradients)");
  if (p->viscous && !(p->mu >= 0 && p->kappa >= 0 && p->cv > 0))
    return fail(MST_EINVAL, "bad viscous coefficients");
  return MST_OK;
}

cudaEvent_t take_event(mst_ctx* c) {
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

int kernel_index(mst_ctx* c, const char* name) {
  for (size_t i = 0; i < c->kname.size(); ++i)
    if (c->kname[i] == name) return (int)i;
  c->kname.push_back(name);
  c->klaunch.push_back(0);
  c->kms.push_back(0.0);
  return (int)c->kname.size() - 1;
}

// brackets one launch with events when profiling is on
struct ProfScope {
  mst_ctx* c;
  int k = -1;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(mst_ctx* ctx, const char* name) : c(ctx) {
    if (!c->profiling) return;
    k = kernel_index(c, name);
    a = take_event(c);
    b = take_event(c);
    cudaEventRecord(a, c->stream);
  }
  ~ProfScope() {
    if (k < 0) return;
    cudaEventRecord(b, c->stream);
    c->pending.push_back({k, a, b});
  }
};

// folds the finished launches into the per-kernel totals
void drain_profile(mst_ctx* c) {
  if (c->pending.empty()) return;
  cudaStreamSynchronize(c->stream);
  for (auto& p : c->pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      c->klaunch[p.kernel] += 1;
      c->kms[p.kernel] += ms;
    }
    c->event_pool.push_back(p.a);
    c->event_pool.push_back(p.b);
  }
  c->pending.clear();
}

// gradient of q (qf: its FP32 copy on the FP32 path); with dt_part it also
// writes the CFL step partials (and dt_cell)
mst_status launch_grad(mst_ctx* c, const double4_32a* q, const float4* qf = nullptr,
                       double* dt_part = nullptr, bool local_dt = false) {
  ProfScope ps(c, c->p.precision == MST_PREC_FP32 ? "k_gradient<f32>" : "k_gradient<f64>");
  const bool f32 = c->p.precision == MST_PREC_FP32;
  if (!f32) qf = nullptr;
  double* dt_cell = (local_dt && !f32) ? c->dt_cell : nullptr;
  float2* dt_cell_ff = (local_dt && f32) ? c->dt_cell_ff : nullptr;
  cudaError_t e = (c->p.precision == MST_PREC_FP64_EXACT)
                      ? mst::exact::launch_gradient_dt(prec_of(c->p), c->dm, q, qf, c->grad,
                                                       c->p.reference_quirks, c->p.cfl,
                                                       dt_cell, dt_cell_ff, dt_part, c->stream)
                      : mst::fast::launch_gradient_dt(prec_of(c->p), c->dm, q, qf, c->grad,
                                                      c->p.reference_quirks, c->p.cfl,
                                                      dt_cell, dt_cell_ff, dt_part, c->stream);
  c->last_launches++;
  if (e != cudaSuccess) return fail(MST_ECUDA, std::string("gradient: ") + cudaGetErrorString(e));
  c->grad_valid = true;
  return MST_OK;
}

mst_status launch_flux(mst_ctx* c, const mst::StepArgs& a) {
  ProfScope ps(c, c->p.precision != MST_PREC_FP32 ? "k_flux_update<f64>"
                  : a.tile_grad                   ? "k_flux_update<f32,tg>"
                                                  : "k_flux_update<f32>");
  cudaError_t e = (c->p.precision == MST_PREC_FP64_EXACT)
                      ? mst::exact::launch_flux_update(prec_of(c->p), c->p.flux, c->p.order,
                                                       c->dm, a, 0, c->stream)
                      : mst::fast::launch_flux_update(prec_of(c->p), c->p.flux, c->p.order,
                                                      c->dm, a, 0, c->stream);
  c->last_launches++;
  if (e != cudaSuccess) return fail(MST_ECUDA, std::string("flux_update: ") + cudaGetErrorString(e));
  return MST_OK;
}

bool pairs(const mst_ctx* c) { return c->p.precision == MST_PREC_FP32; }

// The viscous FP32 float-pair path at 2nd order in the corrected mode forms
// its gradients inside the flux kernel (k_flux_update TG: no gradient pass,
// no gradient through HBM); measured faster there, while the inviscid stage
// keeps the gradient pass (its flux kernel alone is issue-bound, and the
// tile's gradient phases add latency that the pass hides better).  Both
// schedules give bit-identical states.  MSTCFD_FP32_GRADIENT_PASS=1 / =0 in
// the environment forces one schedule, to compare them.
bool tile_grad(const mst_ctx* c) {
  static const int force = [] {
    const char* e = std::getenv("MSTCFD_FP32_GRADIENT_PASS");
    return e ? (e[0] == '1' ? 1 : 0) : -1;
  }();
  const bool can = pairs(c) && c->p.order == 2 && c->p.reference_quirks == 0;
  if (force >= 0) return can && force == 0;
  return can && c->p.viscous;
}

// double copies of the float-pair states (device order) for the entry
// points that read the FP64 buffers
mst_status sync_double_from_pairs(mst_ctx* c) {
  if (!pairs(c)) return MST_OK;
  const int n = c->dm.n_cells, nb = (n + 255) / 256;
  k_from_pairs<<<nb, 256, 0, c->stream>>>(c->qf_old, c->ql_old, nullptr, c->q_old, n);
  k_from_pairs<<<nb, 256, 0, c->stream>>>(c->qf_new, c->ql_new, nullptr, c->q_new, n);
  CU(cudaGetLastError());
  return MST_OK;
}

mst_status sync_pairs_from_double(mst_ctx* c) {
  const int n = c->dm.n_cells, nb = (n + 255) / 256;
  k_to_pairs<<<nb, 256, 0, c->stream>>>(c->q_old, c->qf_old, c->ql_old, n);
  k_to_pairs<<<nb, 256, 0, c->stream>>>(c->q_new, c->qf_new, c->ql_new, n);
  CU(cudaGetLastError());
  return MST_OK;
}

mst::StepArgs base_args(mst_ctx* c) {
  mst::StepArgs a{};
  a.grad = c->grad;
  a.dt = c->p.dt;
  a.quirks = c->p.reference_quirks;
  a.limiter = c->p.limiter;
  mst::set_physics(a, c->p.inlet_q, c->p.viscous, c->p.mu, c->p.lambda, c->p.kappa,
                   c->p.cv);
  return a;
}

// one residual evaluation + update of stage 'stage' from q into qn
// Buffers of one stage: FP64 state q -> qn (q0 = Q^n for stage 1); on the
// FP32 path the float-pair state (qf, ql) -> (qfn, qln) with (q0f, q0l).
struct StageBufs {
  const double4_32a *q = nullptr, *q0 = nullptr;
  double4_32a* qn = nullptr;
  const float4 *qf = nullptr, *ql = nullptr, *q0f = nullptr, *q0l = nullptr;
  float4 *qfn = nullptr, *qln = nullptr;
};

mst_status run_stage(mst_ctx* c, const StageBufs& b, int stage, bool fixed_dt, bool norms,
                     bool keep_residual, bool grad_ready = false) {
  const double4_32a* q = b.q;
  const double4_32a* q0 = b.q0;
  double4_32a* qn = b.qn;
  const float4* qf = pairs(c) ? b.qf : nullptr;
  float4* qfn = pairs(c) ? b.qfn : nullptr;
  const bool tg = tile_grad(c);
  if (c->p.order == 2 && !grad_ready && !tg) {
    mst_status s = launch_grad(c, q, qf);
    if (s) return s;
  }
  mst::StepArgs a = base_args(c);
  a.q = q;
  a.qf = qf;
  a.qfn = qfn;
  a.tile_grad = tg ? 1 : 0;
  if (pairs(c)) {
    a.qlo = b.ql;
    a.qlon = b.qln;
    a.q0f = b.q0f;
    a.q0lo = b.q0l;
    a.dt_ff[0] = (float)c->p.dt;
    a.dt_ff[1] = (float)(c->p.dt - (double)a.dt_ff[0]);
    if (!fixed_dt) a.dt_ff_dev = reinterpret_cast<const float*>(c->scal + 2);
  }
  a.q0 = q0;
  a.qn = qn;
  a.r_out = keep_residual ? c->r : nullptr;
  a.stage = stage;
  if (!fixed_dt) {
    if (c->p.dt_mode == MST_DT_CFL_LOCAL) {
      a.dt_cell = c->dt_cell;
      if (pairs(c)) a.dt_cell_ff = c->dt_cell_ff;
    }
    else a.dt_dev = c->scal;
  }
  a.partials = norms ? c->partials : nullptr;
  return launch_flux(c, a);
}

// step length of the next step into scal[0] (and advances the time); on
// 2nd order the CFL step comes from the stage-0 gradient launch, which is
// then marked ready (*grad_ready)
mst_status compute_dt(mst_ctx* c, const double4_32a* q, double t_end,
                      const float4* qf = nullptr, bool* grad_ready = nullptr) {
  const int nC = c->dm.n_cells;
  int mode = 0;
  if (c->p.dt_mode != MST_DT_FIXED && tile_grad(c)) {
    // no gradient pass on this schedule: the step from the FP32 state alone
    ProfScope ps(c, "k_cfl_dt_pairs");
    cudaError_t e = mst::fast::launch_cfl_dt_pairs(
        c->dm, qf, c->p.cfl, c->p.dt_mode == MST_DT_CFL_LOCAL ? c->dt_cell_ff : nullptr,
        c->dt_part, c->stream);
    c->last_launches++;
    if (e != cudaSuccess) return fail(MST_ECUDA, std::string("cfl_dt: ") + cudaGetErrorString(e));
    mode = 1;
  } else if (c->p.dt_mode != MST_DT_FIXED && c->p.order == 2 && grad_ready) {
    mst_status st = launch_grad(c, q, qf, c->dt_part, c->p.dt_mode == MST_DT_CFL_LOCAL);
    if (st) return st;
    *grad_ready = true;
    mode = 1;
  } else if (c->p.dt_mode != MST_DT_FIXED) {
    ProfScope ps(c, "k_spectral_dt");
    cudaError_t e = (c->p.precision == MST_PREC_FP64_EXACT)
                        ? mst::exact::launch_spectral_dt(prec_of(c->p), c->dm, q, c->p.cfl,
                                                         c->dt_cell, c->dt_part, c->stream)
                        : mst::fast::launch_spectral_dt(prec_of(c->p), c->dm, q, c->p.cfl,
                                                        c->dt_cell, c->dt_part, c->stream);
    c->last_launches++;
    if (e != cudaSuccess) return fail(MST_ECUDA, std::string("spectral_dt: ") + cudaGetErrorString(e));
    if (pairs(c) && c->p.dt_mode == MST_DT_CFL_LOCAL) {
      k_to_pairs1<<<(nC + 255) / 256, 256, 0, c->stream>>>(c->dt_cell, c->dt_cell_ff, nC);
      CU(cudaGetLastError());
    }
    mode = 1;
  }
  ProfScope ps(c, "k_finalize_dt");
  k_finalize_dt<<<1, 1024, 0, c->stream>>>(c->dt_part, (nC + 255) / 256, mode, c->p.dt,
                                            t_end, c->scal);
  c->last_launches++;
  CU(cudaGetLastError());
  return MST_OK;
}

mst_status finalize_norms(mst_ctx* c, bool advance) {
  ProfScope ps(c, "k_finalize_norms");
  k_finalize_norms<<<1, dim3(64, kNormSlots), 0, c->stream>>>(
      c->partials, c->dm.n_tiles, c->dm.n_cells, advance ? 1 : 0, c->scal, c->norms);
  c->last_launches++;
  CU(cudaGetLastError());
  return MST_OK;
}

mst_status read_norms(mst_ctx* c, mst_norms* out) {
  double h[kNormSlots + 2];
  CU(cudaMemcpyAsync(h, c->norms, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  if (out) {
    for (int j = 0; j < 4; ++j) {
      out->linf_change[j] = h[j];
      out->l2_resid[j] = h[4 + j];
    }
    out->mass = h[8];
    out->dt = h[kNormSlots];
    out->time = h[kNormSlots + 1];
  }
  return MST_OK;
}

template <class T>
mst_status dalloc(mst_ctx* c, T** p, size_t bytes) {
  CU(cudaMalloc((void**)p, std::max<size_t>(bytes, 256)));
  c->allocs.push_back(*p);
  return MST_OK;
}

mst_status download_rows(mst_ctx* c, const double4_32a* dev, double* host,
                         size_t stride, const float4* hi = nullptr,
                         const float4* lo = nullptr) {
  const int nC = c->dm.n_cells;
  // device order -> file order with a gather by cell_perm, then one copy
  if (hi)
    k_from_pairs<<<(nC + 255) / 256, 256, 0, c->stream>>>(hi, lo, c->d.cell_perm, c->stage_in, nC);
  else
    k_gather_rows<<<(nC + 255) / 256, 256, 0, c->stream>>>(dev, c->d.cell_perm, c->stage_in, nC);
  CU(cudaGetLastError());
  // contiguous rows (stride 4): one linear copy; a pitched copy of 32-byte
  // rows moves row by row
  if (stride == 4)
    CU(cudaMemcpyAsync(host, c->stage_in, (size_t)nC * 4 * sizeof(double),
                       cudaMemcpyDeviceToHost, c->stream));
  else
    CU(cudaMemcpy2DAsync(host, stride * sizeof(double), c->stage_in, 4 * sizeof(double),
                         4 * sizeof(double), nC, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return MST_OK;
}

}  // namespace

mst_status mst_internal_fail(mst_status s, const std::string& msg) { return fail(s, msg); }

namespace {

// FP64 pipe probe: every thread runs 8 independent fused multiply-add
// chains (x <- x a + b), enough independent work per SM to keep the FP64
// pipe issuing every cycle it can.  With a = 1 - 2^-20 and b small the
// values stay bounded.  The sum is stored so nothing is optimised away.
constexpr int kProbeChains = 8;
__global__ void __launch_bounds__(256) k_probe_dfma(double a, double b, int iters,
                                                    double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double x[kProbeChains];
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) x[k] = 1e-3 * (t & 255) + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) s += x[k];
  out[t] = s;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

const char* mst_last_error(void) { return g_err.c_str(); }
int mst_abi_version(void) { return MSTCFD_ABI_VERSION; }

void mst_params_default(mst_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->flux = MST_FLUX_AUSM;
  p->order = 1;
  p->limiter = MST_LIMITER_NONE;
  p->precision = MST_PREC_FP64_EXACT;
  p->time_scheme = MST_TIME_EULER;
  p->dt_mode = MST_DT_FIXED;
  p->dt = 1.0 / 4e+3;  // 1/STEP_TIME (CONST.h:52, Time.cpp:62)
  p->cfl = 0.5;
  // CONST.h:70-83 as the macros expand: rho 1, u = v = 0, E = 1/286.32*715.8
  p->inlet_q[0] = 1;
  p->inlet_q[1] = 1.0 * 0;
  p->inlet_q[2] = 1.0 * 0;
  p->inlet_q[3] = 1 * (1 / 286.32 * 715.8 + 0.5 * (0 * 0 + 0 * 0));
  p->reference_quirks = 1;
  p->viscous = 0;
  p->mu = 1.7894e-05;              // VISCIDMU (CONST.h:46)
  p->lambda = -0.666667 * 1.7894e-05;  // VISCIDLAMBDA (CONST.h:47)
  p->kappa = 0.0242;               // TEMPK (CONST.h:48)
  p->cv = 715.8;                   // CV (CONST.h:39)
}

mst_status mst_mesh_read_msh(const char* path, mst_mesh** out) {
  if (!path || !out) return fail(MST_EINVAL, "NULL argument");
  *out = nullptr;
  try {
    std::unique_ptr<mst_mesh> m(new mst_mesh);
    std::string err;
    int rc = mst::read_msh(path, &m->host, &err);
    if (rc) return fail(rc == mst::kEInval ? MST_EINVAL : MST_EMESH, err);
    rc = mst::build_layout(m->host, true, &m->lay, &err);
    if (rc) return fail(MST_EMESH, err);
    *out = m.release();
    return MST_OK;
  } catch (const std::bad_alloc&) {
    return fail(MST_ENOMEM, "host allocation failed");
  } catch (...) {
    return fail(MST_EMESH, "mesh read failed");
  }
}

mst_status mst_mesh_create(const mst_mesh_desc* d, mst_mesh** out) {
  if (!d || !out) return fail(MST_EINVAL, "NULL argument");
  *out = nullptr;
  try {
    std::unique_ptr<mst_mesh> m(new mst_mesh);
    std::string err;
    int rc = mst::build_from_arrays(d->n_nodes, d->node_xy, d->n_cells, d->n_faces,
                                    d->face_nodes, d->face_cells, d->n_zones, d->zones,
                                    d->c1_shift, &m->host, &err);
    if (rc) return fail(rc == mst::kEInval ? MST_EINVAL : MST_EMESH, err);
    rc = mst::build_layout(m->host, true, &m->lay, &err);
    if (rc) return fail(MST_EMESH, err);
    *out = m.release();
    return MST_OK;
  } catch (const std::bad_alloc&) {
    return fail(MST_ENOMEM, "host allocation failed");
  } catch (...) {
    return fail(MST_EMESH, "mesh build failed");
  }
}

void mst_mesh_destroy(mst_mesh* m) { delete m; }

mst_status mst_mesh3d_read_msh(const char* path, mst_mesh3d** out) {
  if (!path || !out) return fail(MST_EINVAL, "NULL argument");
  *out = nullptr;
  std::unique_ptr<mst_mesh3d> m(new mst_mesh3d());
  std::string err;
  int rc = mst::read_msh3d(path, &m->host, &err);
  if (rc != mst::kOk) return fail(rc == mst::kEMesh ? MST_EMESH : MST_EINVAL, err);
  *out = m.release();
  return MST_OK;
}

mst_status mst_mesh3d_get_info(const mst_mesh3d* m, mst_mesh3d_info* info) {
  if (!m || !info) return fail(MST_EINVAL, "NULL argument");
  const auto& h = m->host;
  info->n_nodes = h.n_nodes;
  info->n_cells = h.n_cells;
  info->n_faces = h.n_faces;
  info->n_int_faces = h.n_int_faces;
  info->n_zones = (int)h.zone.size() / 4;
  info->n_face_nodes = (int)h.face_nodes.size();
  info->n_cell_faces = (int)h.cell_faces.size();
  info->n_cell_nodes = (int)h.cell_nodes.size();
  info->n_inner = (int)h.inner.size();
  info->n_bond1 = (int)h.bond1.size();
  info->n_bond2 = (int)h.bond2.size();
  return MST_OK;
}

mst_status mst_mesh3d_get_arrays(const mst_mesh3d* m, mst_mesh3d_arrays* a) {
  if (!m || !a) return fail(MST_EINVAL, "NULL argument");
  const auto& h = m->host;
  auto cp = [](auto* dst, const auto& v) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
  };
  cp(a->node_xyz, h.node_xyz);
  cp(a->face_ptr, h.face_ptr);
  cp(a->face_nodes, h.face_nodes);
  cp(a->face_cells, h.face_cells);
  cp(a->face_type, h.face_type);
  cp(a->face_ctr, h.face_ctr);
  cp(a->face_dir, h.face_dir);
  cp(a->face_area, h.face_area);
  cp(a->face_eta0, h.face_eta0);
  cp(a->face_cmd, h.face_cmd);
  cp(a->face_dac, h.face_dac);
  cp(a->face_flag, h.face_flag);
  cp(a->face_flag_set, h.face_flag_set);
  cp(a->cell_ptr, h.cell_ptr);
  cp(a->cell_faces, h.cell_faces);
  cp(a->cell_nb, h.cell_nb);
  cp(a->cell_dof, h.cell_dof);
  cp(a->cell_eta0c, h.cell_eta0c);
  cp(a->cell_ctr, h.cell_ctr);
  cp(a->cell_vol, h.cell_vol);
  cp(a->cell_vol_fixed, h.cell_vol_fixed);
  cp(a->cell_node_ptr, h.cell_node_ptr);
  cp(a->cell_nodes, h.cell_nodes);
  cp(a->inner, h.inner);
  cp(a->bond1, h.bond1);
  cp(a->bond2, h.bond2);
  cp(a->cell_n_lower, h.cell_nL);
  return MST_OK;
}

void mst_mesh3d_destroy(mst_mesh3d* m) { delete m; }

mst_status mst_mesh_get_info(const mst_mesh* m, mst_mesh_info* info) {
  if (!m || !info) return fail(MST_EINVAL, "NULL argument");
  const auto& h = m->host;
  info->n_nodes = h.n_nodes;
  info->n_cells = h.n_cells;
  info->n_faces = h.n_faces;
  info->n_int_faces = h.n_int_faces;
  info->n_zones = h.n_zones();
  info->n_cell_faces = h.cell_ptr.empty() ? 0 : h.cell_ptr.back();
  info->n_inner = (int)h.inner.size();
  info->n_bond1 = (int)h.bond1.size();
  info->n_bond2 = (int)h.bond2.size();
  info->n_tiles = m->lay.n_tiles;
  info->n_borrowed = (int)m->lay.t_bor.size();
  info->n_halo = (int)m->lay.t_halo.size();
  info->n_halo_cells = m->lay.n_halo_cells;
  info->n_halo_cell_faces = m->lay.n_halo_cell_faces;
  return MST_OK;
}

mst_status mst_mesh_get_arrays(const mst_mesh* m, mst_mesh_arrays* a) {
  if (!m || !a) return fail(MST_EINVAL, "NULL argument");
  const auto& h = m->host;
  auto cp = [](auto* dst, const auto& v) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
  };
  cp(a->face_ctr, h.face_ctr);
  cp(a->face_dir, h.face_dir);
  cp(a->face_area, h.face_area);
  cp(a->face_eta0, h.face_eta0);
  cp(a->face_dac, h.face_dac);
  cp(a->face_flag, h.face_flag);
  cp(a->face_cells, h.face_cells);
  cp(a->cell_ptr, h.cell_ptr);
  cp(a->cell_faces, h.cell_faces);
  cp(a->cell_nb, h.cell_nb);
  cp(a->cell_dof, h.cell_dof);
  cp(a->cell_eta0c, h.cell_eta0c);
  cp(a->cell_ctr, h.cell_ctr);
  cp(a->cell_vol, h.cell_vol);
  cp(a->inner, h.inner);
  cp(a->bond1, h.bond1);
  cp(a->bond2, h.bond2);
  cp(a->cell_perm, m->lay.cell_perm);
  cp(a->face_perm, m->lay.face_perm);
  return MST_OK;
}

mst_status mst_ctx_create(const mst_mesh* m, const mst_params* p, mst_ctx** out) {
  if (!m || !out) return fail(MST_EINVAL, "NULL argument");
  *out = nullptr;
  mst_status st = check_params(p);
  if (st) return st;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(MST_ECUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  std::unique_ptr<mst_ctx> c(new (std::nothrow) mst_ctx);
  if (!c) return fail(MST_ENOMEM, "host allocation failed");
  c->mesh = m;
  c->p = *p;
  CU(cudaGetDevice(&c->device));
  CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CU(cudaEventCreate(&c->ev0));
  CU(cudaEventCreate(&c->ev1));
  const auto& L = m->lay;
  DevArrays& d = c->d;
  auto up = [&](auto** dst, const auto& v) -> cudaError_t {
    cudaError_t r = upload(dst, v);
    c->allocs.push_back((void*)*dst);
    return r;
  };
  {
    std::vector<int2> c0c1(L.n_faces);
    for (int i = 0; i < L.n_faces; ++i) c0c1[i] = make_int2(L.f_c0c1[2 * i], L.f_c0c1[2 * i + 1]);
    auto as_d2 = [](const std::vector<double>& v) {
      std::vector<double2> o(v.size() / 2);
      for (size_t i = 0; i < o.size(); ++i) o[i] = make_double2(v[2 * i], v[2 * i + 1]);
      return o;
    };
    auto as_f2 = [](const std::vector<double>& v) {
      std::vector<float2> o(v.size() / 2);
      for (size_t i = 0; i < o.size(); ++i) o[i] = make_float2((float)v[2 * i], (float)v[2 * i + 1]);
      return o;
    };
    CU(up(&d.f_c0c1, c0c1));
    CU(up(&d.f_info, L.f_info));
    CU(up(&d.f_dir, as_d2(L.f_dir)));
    CU(up(&d.f_r0, as_d2(L.f_r0)));
    CU(up(&d.f_r1, as_d2(L.f_r1)));
    CU(up(&d.cf_w, as_d2(L.cf_w)));
    CU(up(&d.f_dir32, as_f2(L.f_dir)));
    CU(up(&d.f_r0_32, as_f2(L.f_r0)));
    CU(up(&d.f_r1_32, as_f2(L.f_r1)));
    CU(up(&d.cf_w32, as_f2(L.cf_w)));
    {
      std::vector<double> cd(2 * L.cf_face.size());
      for (size_t k = 0; k < L.cf_face.size(); ++k) {
        const int fs = L.cf_face[k];
        const int f = fs < 0 ? ~fs : fs;
        cd[2 * k] = fs < 0 ? -L.f_dir[2 * (size_t)f] : L.f_dir[2 * (size_t)f];
        cd[2 * k + 1] = fs < 0 ? -L.f_dir[2 * (size_t)f + 1] : L.f_dir[2 * (size_t)f + 1];
      }
      CU(up(&d.cf_dir, as_d2(cd)));
      CU(up(&d.cf_dir32, as_f2(cd)));
    }
    {
      std::vector<double> fe(L.n_faces);
      std::vector<float> fe32(L.n_faces);
      for (int i = 0; i < L.n_faces; ++i) {
        fe[i] = m->host.face_eta0[L.face_iperm[i]];
        fe32[i] = (float)fe[i];
      }
      CU(up(&d.f_eta, fe));
      CU(up(&d.f_eta32, fe32));
    }
    CU(up(&d.c_vol, L.c_vol));
    for (double v : L.c_vol) c->volumes_ok = c->volumes_ok && std::isfinite(v) && v > 0.0;
    std::vector<double> ivol(L.c_vol.size());
    for (size_t i = 0; i < ivol.size(); ++i) ivol[i] = 1.0 / L.c_vol[i];
    CU(up(&d.c_ivol, ivol));
    std::vector<float2> ivff(ivol.size());
    for (size_t i = 0; i < ivol.size(); ++i) {
      const float h = (float)ivol[i];
      ivff[i] = make_float2(h, (float)(ivol[i] - (double)h));
    }
    CU(up(&d.c_ivol_ff, ivff));
    CU(up(&d.c_ptr, L.c_ptr));
    CU(up(&d.cf_face, L.cf_face));
    CU(up(&d.cf_slot, L.cf_slot));
    CU(up(&d.cf_nb, L.cf_nb));
    CU(up(&d.cf_nb_fix, L.cf_nb_fix));
    CU(up(&d.t_own_ptr, L.t_own_ptr));
    CU(up(&d.t_bor_ptr, L.t_bor_ptr));
    CU(up(&d.t_bor, L.t_bor));
    CU(up(&d.t_halo_ptr, L.t_halo_ptr));
    CU(up(&d.t_halo, L.t_halo));
    CU(up(&d.t_slot_loc, L.t_slot_loc));
    CU(up(&d.cf_nbl, L.cf_nbl));
    CU(up(&d.cell_iperm, L.cell_iperm));
    CU(up(&d.cell_perm, L.cell_perm));
  }
  mst::DevMesh& dm = c->dm;
  dm.n_cells = L.n_cells;
  dm.n_faces = L.n_faces;
  dm.n_tiles = L.n_tiles;
  dm.max_tile_faces = L.max_tile_faces;
  dm.f_c0c1 = d.f_c0c1;
  dm.f_info = d.f_info;
  dm.f_dir = d.f_dir;
  dm.f_r0 = d.f_r0;
  dm.f_r1 = d.f_r1;
  dm.f_dir32 = d.f_dir32;
  dm.f_r0_32 = d.f_r0_32;
  dm.f_r1_32 = d.f_r1_32;
  dm.f_eta = d.f_eta;
  dm.f_eta32 = d.f_eta32;
  dm.c_vol = d.c_vol;
  dm.c_ivol = d.c_ivol;
  dm.c_ivol_ff = d.c_ivol_ff;
  dm.c_ptr = d.c_ptr;
  dm.cf_face = d.cf_face;
  dm.cf_slot = d.cf_slot;
  dm.cf_nb = d.cf_nb;
  dm.cf_nb_fix = d.cf_nb_fix;
  dm.cf_w = d.cf_w;
  dm.cf_w32 = d.cf_w32;
  dm.cf_dir = d.cf_dir;
  dm.cf_dir32 = d.cf_dir32;
  dm.t_own_ptr = d.t_own_ptr;
  dm.t_bor_ptr = d.t_bor_ptr;
  dm.t_bor = d.t_bor;
  dm.t_halo_ptr = d.t_halo_ptr;
  dm.t_halo = d.t_halo;
  dm.t_slot_loc = d.t_slot_loc;
  dm.cf_nbl = d.cf_nbl;
  dm.max_halo = L.max_halo;
  dm.deg3 = 1;
  for (int i = 0; i <= L.n_cells && dm.deg3; ++i) dm.deg3 = L.c_ptr[i] == 3 * i;
  const size_t nC = L.n_cells, nB = (nC + 255) / 256;
  const size_t qbytes = nC * sizeof(double4_32a);
  if ((st = dalloc(c.get(), &c->q_old, qbytes)) || (st = dalloc(c.get(), &c->q_new, qbytes)) ||
      (st = dalloc(c.get(), &c->q_stage, qbytes)) || (st = dalloc(c.get(), &c->r, qbytes)) ||
      (st = dalloc(c.get(), &c->stage_in, qbytes)) ||
      (st = dalloc(c.get(), &c->qf_old, nC * sizeof(float4))) ||
      (st = dalloc(c.get(), &c->qf_new, nC * sizeof(float4))) ||
      (st = dalloc(c.get(), &c->qf_stage, nC * sizeof(float4))) ||
      (st = dalloc(c.get(), &c->ql_old, nC * sizeof(float4))) ||
      (st = dalloc(c.get(), &c->ql_new, nC * sizeof(float4))) ||
      (st = dalloc(c.get(), &c->ql_stage, nC * sizeof(float4))) ||
      (st = dalloc(c.get(), (char**)&c->grad, nC * 8 * sizeof(double))) ||
      (st = dalloc(c.get(), &c->partials,
                   std::max<size_t>(L.n_tiles, nB) * kNormSlots * sizeof(double))) ||
      (st = dalloc(c.get(), &c->dt_part, nB * sizeof(double))) ||
      (st = dalloc(c.get(), &c->dt_cell, nC * sizeof(double))) ||
      (st = dalloc(c.get(), &c->dt_cell_ff, nC * sizeof(float2))) ||
      (st = dalloc(c.get(), &c->scal, 4 * sizeof(double))) ||
      (st = dalloc(c.get(), &c->norms, (kNormSlots + 2) * sizeof(double))))
    return st;
  CU(cudaMemset(c->q_old, 0, qbytes));
  CU(cudaMemset(c->q_new, 0, qbytes));
  CU(cudaMemset(c->r, 0, qbytes));
  CU(cudaMemset(c->scal, 0, 4 * sizeof(double)));
  CU(cudaMemset(c->norms, 0, (kNormSlots + 2) * sizeof(double)));
  CU(cudaDeviceSynchronize());
  *out = c.release();
  return MST_OK;
}

mst_status mst_ctx_destroy(mst_ctx* c) {
  if (!c) return MST_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  mst_io_release(c);
  for (void* p : c->allocs) cudaFree(p);
  for (auto& p : c->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t e : c->event_pool) cudaEventDestroy(e);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  release_pipe(c);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return MST_OK;
}

mst_status mst_ctx_set_params(mst_ctx* c, const mst_params* p) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  mst_status st = check_params(p);
  if (st) return st;
  const bool was = pairs(c);
  const bool to_pairs = p->precision == MST_PREC_FP32 && !was;
  if (was && p->precision != MST_PREC_FP32) {  // the FP64 buffers were not kept
    mst_status s = sync_double_from_pairs(c);
    if (s) return s;
  }
  c->p = *p;
  c->grad_valid = false;
  if (to_pairs) {
    mst_status s = sync_pairs_from_double(c);
    if (s) return s;
  }
  CU(cudaStreamSynchronize(c->stream));
  return MST_OK;
}

mst_status mst_set_dt(mst_ctx* c, double dt) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  if (!(dt >= 0)) return fail(MST_EINVAL, "dt must be >= 0");
  c->p.dt = dt;
  return MST_OK;
}

mst_status mst_set_state(mst_ctx* c, const double* q, size_t stride) {
  if (!c || !q) return fail(MST_EINVAL, "NULL argument");
  if (stride < 4) return fail(MST_EINVAL, "stride must be >= 4 doubles");
  const int nC = c->dm.n_cells;
  if (stride == 4)
    CU(cudaMemcpyAsync(c->stage_in, q, (size_t)nC * 4 * sizeof(double), cudaMemcpyHostToDevice,
                       c->stream));
  else
    CU(cudaMemcpy2DAsync(c->stage_in, 4 * sizeof(double), q, stride * sizeof(double),
                         4 * sizeof(double), nC, cudaMemcpyHostToDevice, c->stream));
  k_gather_rows<<<(nC + 255) / 256, 256, 0, c->stream>>>(c->stage_in, c->d.cell_iperm,
                                                           c->q_old, nC);
  CU(cudaGetLastError());
  CU(cudaMemcpyAsync(c->q_new, c->q_old, (size_t)nC * sizeof(double4_32a),
                     cudaMemcpyDeviceToDevice, c->stream));
  if (pairs(c)) {
    mst_status s = sync_pairs_from_double(c);
    if (s) return s;
  }
  CU(cudaStreamSynchronize(c->stream));
  c->grad_valid = false;
  return MST_OK;
}

mst_status mst_get_state(mst_ctx* c, double* q, size_t stride) {
  if (!c || !q) return fail(MST_EINVAL, "NULL argument");
  if (stride < 4) return fail(MST_EINVAL, "stride must be >= 4 doubles");
  if (pairs(c)) return download_rows(c, nullptr, q, stride, c->qf_old, c->ql_old);
  return download_rows(c, c->q_old, q, stride);
}

mst_status mst_get_new_state(mst_ctx* c, double* q, size_t stride) {
  if (!c || !q) return fail(MST_EINVAL, "NULL argument");
  if (stride < 4) return fail(MST_EINVAL, "stride must be >= 4 doubles");
  if (pairs(c)) return download_rows(c, nullptr, q, stride, c->qf_new, c->ql_new);
  return download_rows(c, c->q_new, q, stride);
}

mst_status mst_get_residual(mst_ctx* c, double* r, size_t stride) {
  if (!c || !r) return fail(MST_EINVAL, "NULL argument");
  if (stride < 4) return fail(MST_EINVAL, "stride must be >= 4 doubles");
  return download_rows(c, c->r, r, stride);
}

mst_status mst_solve(mst_ctx* c) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  c->last_launches = 0;
  CU(cudaEventRecord(c->ev0, c->stream));
  StageBufs b;
  b.q = c->q_old;
  b.qn = c->q_new;
  b.qf = c->qf_old;
  b.ql = c->ql_old;
  b.qfn = c->qf_new;
  b.qln = c->ql_new;
  mst_status s = run_stage(c, b, 0, true, true, true);
  if (s) return s;
  if ((s = finalize_norms(c, false))) return s;
  CU(cudaEventRecord(c->ev1, c->stream));
  c->timed = true;
  CU(cudaStreamSynchronize(c->stream));
  drain_profile(c);
  return MST_OK;
}

mst_status mst_update_new_to_old(mst_ctx* c) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  CU(cudaMemcpyAsync(c->q_old, c->q_new, (size_t)c->dm.n_cells * sizeof(double4_32a),
                     cudaMemcpyDeviceToDevice, c->stream));
  if (pairs(c)) {
    CU(cudaMemcpyAsync(c->qf_old, c->qf_new, (size_t)c->dm.n_cells * sizeof(float4),
                       cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaMemcpyAsync(c->ql_old, c->ql_new, (size_t)c->dm.n_cells * sizeof(float4),
                       cudaMemcpyDeviceToDevice, c->stream));
  }
  CU(cudaStreamSynchronize(c->stream));
  c->grad_valid = false;
  return MST_OK;
}

mst_status mst_get_face_flux(mst_ctx* c, double* f) {
  if (!c || !f) return fail(MST_EINVAL, "NULL argument");
  const int nF = c->dm.n_faces;
  if (!c->flux) {
    mst_status s = dalloc(c, &c->flux, (size_t)nF * 8 * sizeof(double));
    if (s) return s;
  }
  if (pairs(c)) {
    mst_status s = sync_double_from_pairs(c);
    if (s) return s;
  }
  if (c->p.order == 2 && !c->grad_valid) {
    mst_status s = launch_grad(c, c->q_old);
    if (s) return s;
  }
  mst::StepArgs a = base_args(c);
  a.q = c->q_old;
  cudaError_t e = (c->p.precision == MST_PREC_FP64_EXACT)
                      ? mst::exact::launch_face_flux(prec_of(c->p), c->p.flux, c->p.order, c->dm, a,
                                                     c->flux, c->stream)
                      : mst::fast::launch_face_flux(prec_of(c->p), c->p.flux, c->p.order, c->dm, a,
                                                    c->flux, c->stream);
  if (e != cudaSuccess) return fail(MST_ECUDA, std::string("face_flux: ") + cudaGetErrorString(e));
  std::vector<double> h((size_t)nF * 8);
  CU(cudaMemcpyAsync(h.data(), c->flux, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                     c->stream));
  CU(cudaStreamSynchronize(c->stream));
  const auto& L = c->mesh->lay;
  for (int i = 0; i < nF; ++i)
    std::memcpy(f + 8 * (size_t)i, h.data() + 8 * (size_t)L.face_perm[i], 8 * sizeof(double));
  return MST_OK;
}

mst_status mst_get_gradient(mst_ctx* c, double* g) {
  if (!c || !g) return fail(MST_EINVAL, "NULL argument");
  if (c->p.order != 2) return fail(MST_EINVAL, "gradients exist for order 2 only");
  if (pairs(c) && !c->grad_valid) {
    mst_status s = sync_double_from_pairs(c);
    if (s) return s;
  }
  if (!c->grad_valid) {
    mst_status s = launch_grad(c, c->q_old);
    if (s) return s;
  }
  const int nC = c->dm.n_cells;
  const auto& L = c->mesh->lay;
  if (c->p.precision == MST_PREC_FP32) {
    std::vector<float> h((size_t)nC * 8);
    CU(cudaMemcpyAsync(h.data(), c->grad, h.size() * sizeof(float), cudaMemcpyDeviceToHost,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < nC; ++i)
      for (int k = 0; k < 8; ++k) g[8 * (size_t)i + k] = h[8 * (size_t)L.cell_perm[i] + k];
  } else {
    std::vector<double> h((size_t)nC * 8);
    CU(cudaMemcpyAsync(h.data(), c->grad, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < nC; ++i)
      std::memcpy(g + 8 * (size_t)i, h.data() + 8 * (size_t)L.cell_perm[i], 8 * sizeof(double));
  }
  return MST_OK;
}

}  // extern "C"

namespace {

// nsteps steps of the configured scheme enqueued on the context's stream
// (no host synchronisation); norms of the last step into c->norms when
// last_norms is set
mst_status enqueue_steps(mst_ctx* c, int nsteps, double t_end, bool last_norms = true) {
  for (int s = 0; s < nsteps; ++s) {
    // norms (per-tile partials + one reduction) on the last step only
    const bool norms = last_norms && (s == nsteps - 1);
    bool grad_ready = false;
    mst_status st = compute_dt(c, c->q_old, t_end, c->qf_old, &grad_ready);
    if (st) return st;
    StageBufs b0;
    b0.q = c->q_old;
    b0.qf = c->qf_old;
    b0.ql = c->ql_old;
    if (c->p.time_scheme == MST_TIME_EULER) {
      b0.qn = c->q_new;
      b0.qfn = c->qf_new;
      b0.qln = c->ql_new;
      st = run_stage(c, b0, 0, false, norms, false, grad_ready);
    } else {
      b0.qn = c->q_stage;
      b0.qfn = c->qf_stage;
      b0.qln = c->ql_stage;
      st = run_stage(c, b0, 0, false, false, false, grad_ready);
      StageBufs b1;
      b1.q = c->q_stage;
      b1.qf = c->qf_stage;
      b1.ql = c->ql_stage;
      b1.q0 = c->q_old;
      b1.q0f = c->qf_old;
      b1.q0l = c->ql_old;
      b1.qn = c->q_new;
      b1.qfn = c->qf_new;
      b1.qln = c->ql_new;
      if (!st) st = run_stage(c, b1, 1, false, norms, false);
    }
    if (st) return st;
    if (norms && (st = finalize_norms(c, true))) return st;
    std::swap(c->q_old, c->q_new);
    std::swap(c->qf_old, c->qf_new);
    std::swap(c->ql_old, c->ql_new);
  }
  return MST_OK;
}

// ---- host-buffer pipeline ----
__global__ void k_copy_doubles(const double* __restrict__ src, double* __restrict__ dst, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

__global__ void k_load_rows(const double4_32a* __restrict__ src, const int* __restrict__ iperm,
                            double4_32a* __restrict__ q, float4* __restrict__ hi,
                            float4* __restrict__ lo, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4_32a v = src[iperm[i]];
  if (q) q[i] = v;
  if (hi) {
    const float4 h = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
    hi[i] = h;
    lo[i] = make_float4((float)(v.x - (double)h.x), (float)(v.y - (double)h.y),
                        (float)(v.z - (double)h.z), (float)(v.w - (double)h.w));
  }
}

void release_pipe(mst_ctx* c) {
  mst_ctx::HostPipe& P = c->pipe;
  if (P.in) cudaStreamSynchronize(P.in);
  if (P.out) cudaStreamSynchronize(P.out);
  for (int k = 0; k < 2; ++k) {
    cudaFree(P.slot_in[k]);
    cudaFree(P.slot_out[k]);
    for (cudaEvent_t e : {P.in_ready[k], P.in_free[k], P.out_ready[k], P.out_free[k]})
      if (e) cudaEventDestroy(e);
  }
  cudaFree(P.job_norms);
  if (P.in) cudaStreamDestroy(P.in);
  if (P.out) cudaStreamDestroy(P.out);
  P = mst_ctx::HostPipe{};
}

mst_status ensure_pipe(mst_ctx* c, int n_jobs) {
  mst_ctx::HostPipe& P = c->pipe;
  const size_t qbytes = (size_t)c->dm.n_cells * sizeof(double4_32a);
  if (!P.in) {
    CU(cudaStreamCreateWithFlags(&P.in, cudaStreamNonBlocking));
    CU(cudaStreamCreateWithFlags(&P.out, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
      CU(cudaMalloc((void**)&P.slot_in[k], std::max<size_t>(qbytes, 256)));
      CU(cudaMalloc((void**)&P.slot_out[k], std::max<size_t>(qbytes, 256)));
      for (cudaEvent_t* e : {&P.in_ready[k], &P.in_free[k], &P.out_ready[k], &P.out_free[k]})
        CU(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
  }
  if (n_jobs > P.cap) {
    cudaFree(P.job_norms);
    P.job_norms = nullptr;
    P.cap = 0;
    CU(cudaMalloc((void**)&P.job_norms, sizeof(double) * (kNormSlots + 2) * (size_t)n_jobs));
    P.cap = n_jobs;
  }
  return MST_OK;
}

}  // namespace

extern "C" {

mst_status mst_step_host_jobs(mst_ctx* c, int n_jobs, const double* const* q_in,
                              double* const* q_out, int nsteps) {
  if (!c || n_jobs < 0 || nsteps < 1 || (n_jobs > 0 && (!q_in || !q_out)))
    return fail(MST_EINVAL, "NULL argument, n_jobs < 0 or nsteps < 1");
  for (int j = 0; j < n_jobs; ++j)
    if (!q_in[j] || !q_out[j]) return fail(MST_EINVAL, "NULL job buffer");
  if (n_jobs == 0) return MST_OK;
  mst_status st = ensure_pipe(c, n_jobs);
  if (st) return st;
  mst_ctx::HostPipe& P = c->pipe;
  const int nC = c->dm.n_cells;
  const size_t qbytes = (size_t)nC * sizeof(double4_32a);
  const int nb = (nC + 255) / 256;
  const bool fp32 = pairs(c);
  c->last_launches = 0;
  CU(cudaEventRecord(c->ev0, c->stream));
  // no slot is in use before the first jobs
  for (int k = 0; k < 2; ++k) {
    CU(cudaEventRecord(P.in_free[k], c->stream));
    CU(cudaEventRecord(P.out_free[k], P.out));
  }
  for (int j = 0; j < n_jobs; ++j) {
    const int k = j & 1;
    // in: host -> slot (after the slot's previous job was loaded)
    CU(cudaStreamWaitEvent(P.in, P.in_free[k], 0));
    CU(cudaMemcpyAsync(P.slot_in[k], q_in[j], qbytes, cudaMemcpyHostToDevice, P.in));
    CU(cudaEventRecord(P.in_ready[k], P.in));
    // compute: slot -> state (device order; float pairs on the FP32 path)
    CU(cudaStreamWaitEvent(c->stream, P.in_ready[k], 0));
    k_load_rows<<<nb, 256, 0, c->stream>>>(P.slot_in[k], c->d.cell_iperm,
                                            fp32 ? nullptr : c->q_old,
                                            fp32 ? c->qf_old : nullptr,
                                            fp32 ? c->ql_old : nullptr, nC);
    CU(cudaGetLastError());
    CU(cudaEventRecord(P.in_free[k], c->stream));
    c->grad_valid = false;
    st = enqueue_steps(c, nsteps, 0.0);
    if (st) return st;
    // the job's norms kept for the divergence check: a one-warp copy (a
    // device-to-device cudaMemcpyAsync would go through a copy engine and
    // could queue behind the other jobs' 64 MB host transfers)
    k_copy_doubles<<<1, 32, 0, c->stream>>>(c->norms, P.job_norms + (size_t)j * (kNormSlots + 2),
                                            kNormSlots + 2);
    CU(cudaGetLastError());
    // state -> out slot in file order (after the slot's previous job left)
    CU(cudaStreamWaitEvent(c->stream, P.out_free[k], 0));
    if (fp32)
      k_from_pairs<<<nb, 256, 0, c->stream>>>(c->qf_old, c->ql_old, c->d.cell_perm,
                                               P.slot_out[k], nC);
    else
      k_gather_rows<<<nb, 256, 0, c->stream>>>(c->q_old, c->d.cell_perm, P.slot_out[k], nC);
    CU(cudaGetLastError());
    c->last_launches += 3;
    CU(cudaEventRecord(P.out_ready[k], c->stream));
    // out: slot -> host
    CU(cudaStreamWaitEvent(P.out, P.out_ready[k], 0));
    CU(cudaMemcpyAsync(q_out[j], P.slot_out[k], qbytes, cudaMemcpyDeviceToHost, P.out));
    CU(cudaEventRecord(P.out_free[k], P.out));
  }
  CU(cudaEventRecord(c->ev1, P.out));
  c->timed = true;
  CU(cudaStreamSynchronize(P.out));
  CU(cudaStreamSynchronize(c->stream));
  drain_profile(c);
  // the context's state is the last job's result; every job's last-step
  // norms decide divergence as in mst_step
  std::vector<double> h((size_t)n_jobs * (kNormSlots + 2));
  CU(cudaMemcpy(h.data(), P.job_norms, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
  if (c->volumes_ok) {
    for (int j = 0; j < n_jobs; ++j) {
      const double* n = h.data() + (size_t)j * (kNormSlots + 2);
      bool finite = std::isfinite(n[8]);
      for (int q = 4; q < 8; ++q) finite = finite && std::isfinite(n[q]);
      if (!finite)
        return fail(MST_EDIVERGED, "mst_step_host_jobs: job " + std::to_string(j) +
                                       ": the residual or the mass is not finite");
    }
  }
  return MST_OK;
}

mst_status mst_step(mst_ctx* c, int nsteps, double t_end, mst_norms* last) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  if (nsteps < 0) return fail(MST_EINVAL, "nsteps must be >= 0");
  c->last_launches = 0;
  CU(cudaEventRecord(c->ev0, c->stream));
  {
    mst_status st = enqueue_steps(c, nsteps, t_end);
    if (st) return st;
  }
  CU(cudaEventRecord(c->ev1, c->stream));
  c->timed = true;
  c->grad_valid = false;
  drain_profile(c);
  if (nsteps == 0) {
    if (last) return read_norms(c, last);
    CU(cudaStreamSynchronize(c->stream));
    return MST_OK;
  }
  // the last step's norms: on a mesh of finite positive volumes, a
  // residual or mass that is not finite means the state left the physical
  // range (NaN, non-positive density or pressure)
  mst_norms n{};
  mst_status st = read_norms(c, &n);
  if (st) return st;
  if (last) *last = n;
  bool finite = std::isfinite(n.mass);
  for (int j = 0; j < 4; ++j) finite = finite && std::isfinite(n.l2_resid[j]);
  if (!finite && c->volumes_ok)
    return fail(MST_EDIVERGED, "mst_step: the residual or the mass is not finite (NaN or "
                               "non-positive density or pressure)");
  return MST_OK;
}

mst_status mst_profile_enable(mst_ctx* c, int on) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  drain_profile(c);
  c->profiling = on != 0;
  return MST_OK;
}

mst_status mst_profile_reset(mst_ctx* c) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  drain_profile(c);
  c->kname.clear();
  c->klaunch.clear();
  c->kms.clear();
  return MST_OK;
}

int mst_profile_count(mst_ctx* c) {
  if (!c) return 0;
  drain_profile(c);
  return (int)c->kname.size();
}

mst_status mst_profile_get(mst_ctx* c, int i, char* name, size_t name_len,
                           int* launches, double* total_ms) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  drain_profile(c);
  if (i < 0 || i >= (int)c->kname.size()) return fail(MST_EINVAL, "no such kernel");
  if (name && name_len) {
    std::strncpy(name, c->kname[i].c_str(), name_len - 1);
    name[name_len - 1] = 0;
  }
  if (launches) *launches = c->klaunch[i];
  if (total_ms) *total_ms = c->kms[i];
  return MST_OK;
}

mst_status mst_host_alloc(size_t bytes, void** out) {
  if (!out) return fail(MST_EINVAL, "NULL argument");
  *out = nullptr;
  CU(cudaHostAlloc(out, std::max<size_t>(bytes, 1), cudaHostAllocDefault));
  return MST_OK;
}

mst_status mst_host_free(void* p) {
  if (p) CU(cudaFreeHost(p));
  return MST_OK;
}

mst_status mst_set_device(int device) {
  int n = 0;
  CU(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(MST_EINVAL, "no such device");
  CU(cudaSetDevice(device));
  return MST_OK;
}

mst_status mst_device_count(int* n) {
  if (!n) return fail(MST_EINVAL, "NULL argument");
  *n = 0;
  cudaError_t e = cudaGetDeviceCount(n);
  if (e != cudaSuccess) {
    *n = 0;
    return fail(MST_ECUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
  }
  return MST_OK;
}

mst_status mst_probe_fp64_rate(double* dfma_per_s) {
  if (!dfma_per_s) return fail(MST_EINVAL, "NULL argument");
  *dfma_per_s = 0.0;
  int dev = 0, sms = 0;
  CU(cudaGetDevice(&dev));
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int threads = 256, blocks = sms * 8, iters = 4096;
  double* out = nullptr;
  CU(cudaMalloc((void**)&out, sizeof(double) * (size_t)threads * blocks));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first warms up
    cudaEventRecord(e0, 0);
    k_probe_dfma<<<blocks, threads>>>(1.0 - 0x1p-20, 1e-9, iters, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
    cudaEventRecord(e1, 0);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return fail(MST_ECUDA, std::string("fp64 probe: ") + cudaGetErrorString(e));
  if (!(best > 0.f)) return fail(MST_ECUDA, "fp64 probe: no timing");
  *dfma_per_s = (double)threads * blocks * iters * kProbeChains / (best * 1e-3);
  return MST_OK;
}

mst_status mst_get_time(mst_ctx* c, double* t) {
  if (!c || !t) return fail(MST_EINVAL, "NULL argument");
  double h[4];
  CU(cudaMemcpyAsync(h, c->scal, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  *t = h[1];
  return MST_OK;
}

mst_status mst_last_timing(mst_ctx* c, double* ms, int* launches) {
  if (!c) return fail(MST_EINVAL, "NULL context");
  if (!c->timed) return fail(MST_EINVAL, "nothing timed yet");
  CU(cudaEventSynchronize(c->ev1));
  float f = 0;
  CU(cudaEventElapsedTime(&f, c->ev0, c->ev1));
  if (ms) *ms = f;
  if (launches) *launches = c->last_launches;
  return MST_OK;
}

}  // extern "C"
