// Batched steady solves: many independent cases (meshes with their own
// inflow state and transport coefficients) iterated together to a
// residual tolerance by matrix-free LU-SGS (implicit.inc).
//
// The cases are joined into one disjoint-union mesh (mst::build_union):
// each case keeps its own Morton ordering and occupies a contiguous range
// of device cells, every face carries its case id, so the residual kernels
// of the explicit path run unchanged over all cases at once and take the
// inflow state and viscosity of each face's case from a table.  Per
// iteration: gradient, residual, per-case norms and CFL (one block per
// case), then the forward and backward LU-SGS sweeps, one launch per
// colour of the cell adjacency.  graph_iters iterations are captured once
// into a CUDA graph and replayed until every case has converged.  The
// sweep block size is chosen at creation by timing the candidates (the
// sweeps give the same result for any block size).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ctx.hpp"

namespace {

#define B_CU(call)                                                             \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return mst_internal_fail(MST_ECUDA, std::string(#call) + ": " +          \
                                              cudaGetErrorString(e_));         \
  } while (0)

__global__ void k_batch_gather(const double4_32a* __restrict__ src,
                               const int* __restrict__ idx, double4_32a* __restrict__ dst,
                               int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[idx[i]];
}
// Per-case progress of a case that (re)starts: all cases with `all`, else
// those flagged in `flag` (restarts from the fallback states, which also
// un-count a retired case and start its iteration numbers at *iter).
struct CaseProgress {
  double *cfl, *l2_win, *stall_best;
  int *conv_iter, *diverged, *frozen, *stall_best_it, *restart_it, *n_conv, *iter;
};
__global__ void k_batch_reset(int n_cases, double cfl0, CaseProgress p, const int* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int it = flag ? *p.iter : 0;
  if (i < n_cases && (!flag || flag[i])) {
    if (flag && p.conv_iter[i] >= 0) atomicSub(p.n_conv, 1);
    p.cfl[i] = cfl0;
    p.conv_iter[i] = -1;
    p.diverged[i] = 0;
    p.frozen[i] = 0;
    p.l2_win[i] = 0.0;
    p.stall_best[i] = 1e300;
    p.stall_best_it[i] = it;
    p.restart_it[i] = it;
  }
  if (!flag && i == 0) {
    *p.n_conv = 0;
    *p.iter = 0;
  }
}

// the fallback state of every cell of a flagged case into both state
// buffers (and their FP32 copies where they exist)
__global__ void k_restart_cells(int n, const int* __restrict__ c_case, const int* __restrict__ flag,
                                const double4_32a* __restrict__ q_fb, double4_32a* q0,
                                double4_32a* q1, float4* f0, float4* f1) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n || !flag[c_case[c]]) return;
  const double4_32a v = q_fb[c];
  q0[c] = v;
  q1[c] = v;
  const float4 f = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
  if (f0) f0[c] = f;
  if (f1) f1[c] = f;
}

}  // namespace

struct mst_batch {
  mst_mesh* mesh = nullptr;  // the union mesh (owned)
  mst_ctx* ctx = nullptr;    // context on it (owned)
  int n_cases = 0;
  int n_colors = 0;
  int threads = 128;
  mst_implicit_params ip{};
  std::vector<int> color_off;    // [n_colors + 1] into color_cells
  std::vector<int> color_file;   // colour of every union cell, file order
  int* color = nullptr;          // device order
  int* color_cells = nullptr;
  int* c_case = nullptr;
  int* case_first = nullptr;
  double* case_tab = nullptr;
  float* case_tab_f = nullptr;
  double *cfl = nullptr, *first = nullptr, *last = nullptr;
  int *conv_iter = nullptr, *n_conv = nullptr, *iter = nullptr;
  int* diverged = nullptr;       // per case: retired with a non-finite L2
  int* frozen = nullptr;         // per-case limiter-freezing state
  double* l2_win = nullptr;      // per-case L2 at the last freezing check
  double* own_first = nullptr;   // per-case L2 of this run's first iteration
  double* frz_best = nullptr;    // per-case best L2 since its limiter froze
  int* frz_best_it = nullptr;
  double* stall_best = nullptr;  // per-case best L2 of the stall test
  int* stall_best_it = nullptr;
  int* restart_it = nullptr;     // per-case iteration of its (re)start
  int* restart_flag = nullptr;   // per-case flags of one restart call
  double4_32a* q_fb = nullptr;   // fallback states (device order), or nullptr
  bool has_fb = false;
  std::vector<int> restart_iter; // host: per case its restart iteration or -1
  // compaction: once most cases have converged, the residual kernels visit
  // the tiles and the sweeps the cells of unconverged cases only
  std::vector<int> c_case_h;     // case of every device cell
  std::vector<int> color_cells_h;
  int* tile_list = nullptr;      // device [n_tiles]
  int* act_cells = nullptr;      // device [n_cells]: per colour, active cells
  std::vector<int> act_off;      // [n_colors + 1] into act_cells
  bool compact = false;          // lists in use
  long long list_cells = 0;      // cells of the cases the lists hold
  void* phi = nullptr;           // recorded limiter ratios [n_faces][2][4]
  double4_32a* dq = nullptr;
  double* diag = nullptr;
  float4* dqf = nullptr;         // FP32 sweeps: dQ* / dQ in FP32
  bool sweep32 = false;
  bool first_fixed = false;      // reference L2s set by mst_batch_set_l2_ref
  double* norm_part = nullptr;   // [n_cases][8] partial L2 sums
  int cur = 0;                   // which of ctx->q_old / q_new holds Q
  // mixed precision: each case evaluates the FP32 residual (FP32 state
  // copy, FP32 gradient) until it is ready for the FP64 one; lo is set
  // while any case is still in the FP32 phase (case_lo / lo_h: per case)
  bool lo = false;
  void* grad32 = nullptr;
  int* case_lo = nullptr;
  std::vector<int> lo_h;
  // phase-switch bookkeeping: per case the best FP32-phase L2 and when
  std::vector<double> lo_best;
  std::vector<int> lo_best_it;
  bool tuned = false;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [FP64 phase, FP32 phase]
  int graph_iters[2] = {0, 0};
  int graph_cur[2] = {0, 0};     // the buffer the captured iterations start from
  std::vector<void*> allocs;
};

namespace {

template <class T>
mst_status balloc(mst_batch* b, T** p, size_t bytes) {
  B_CU(cudaMalloc((void**)p, std::max<size_t>(bytes, 256)));
  b->allocs.push_back(*p);
  return MST_OK;
}

template <class T>
mst_status bupload(mst_batch* b, T** p, const std::vector<T>& v) {
  mst_status s = balloc(b, p, v.size() * sizeof(T));
  if (s) return s;
  if (!v.empty()) B_CU(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return MST_OK;
}

double4_32a* qbuf(mst_batch* b, int which) { return which ? b->ctx->q_new : b->ctx->q_old; }
// FP32 copy of the state, kept where an FP32 residual reads it
float4* qfbuf(mst_batch* b, int which) {
  if (b->ctx->p.precision != MST_PREC_FP32 && !b->lo && !b->sweep32) return nullptr;
  return which ? b->ctx->qf_new : b->ctx->qf_old;
}

bool exact(const mst_batch* b) { return b->ctx->p.precision == MST_PREC_FP64_EXACT; }

// the residual R(Q) of the current state into ctx->r for the cases that
// dm admits, in the FP32 (lo) or the solve's own precision
mst_status residual_pass(mst_batch* b, int which, bool lo, const mst::DevMesh& dm) {
  mst_ctx* c = b->ctx;
  const int prec = lo ? MST_PREC_FP32 : c->p.precision;
  void* grad = lo ? b->grad32 : c->grad;
  cudaStream_t s = c->stream;
  const double4_32a* q = qbuf(b, which);
  const float4* qf = qfbuf(b, which);
  cudaError_t e = cudaSuccess;
  if (c->p.order == 2) {
    if (exact(b) && !lo) e = mst::exact::launch_gradient(prec, dm, q, grad, 0, s);
    else if (qf)
      e = mst::fast::launch_gradient_dt(prec, dm, q, qf, grad, 0, 0.0, nullptr, nullptr,
                                        nullptr, s);
    else e = mst::fast::launch_gradient(prec, dm, q, grad, 0, s);
    if (e != cudaSuccess)
      return mst_internal_fail(MST_ECUDA, std::string("gradient: ") + cudaGetErrorString(e));
  }
  mst::StepArgs a{};
  a.q = q;
  a.qf = qf;
  a.grad = grad;
  a.r_out = c->r;
  a.quirks = 0;
  a.limiter = c->p.limiter;
  mst::set_physics(a, c->p.inlet_q, c->p.viscous, c->p.mu, c->p.lambda, c->p.kappa, c->p.cv);
  a.case_tab = b->case_tab;
  a.case_tab_f = b->case_tab_f;
  if (b->ip.freeze_tol > 0 && c->p.order == 2 && c->p.limiter != MST_LIMITER_NONE && !lo) {
    a.case_frozen = b->frozen;
    a.phi = b->phi;
  }
  e = (exact(b) && !lo)
          ? mst::exact::launch_flux_update(prec, c->p.flux, c->p.order, dm, a, 0, s)
          : mst::fast::launch_flux_update(prec, c->p.flux, c->p.order, dm, a, 0, s);
  if (e != cudaSuccess)
    return mst_internal_fail(MST_ECUDA, std::string("residual: ") + cudaGetErrorString(e));
  return MST_OK;
}

// the residual R(Q) of the current state into ctx->r: while some case is in
// the FP32 phase, one pass per phase, each skipping the other phase's cases
// (a case's cells, gradient and faces never mix the two precisions)
mst_status enqueue_residual(mst_batch* b, int which) {
  if (!b->lo) return residual_pass(b, which, false, b->ctx->dm);
  mst::DevMesh dm = b->ctx->dm;
  dm.case_lo = b->case_lo;
  dm.lo_want = 1;
  mst_status st = residual_pass(b, which, true, dm);
  if (st) return st;
  dm.lo_want = 0;
  return residual_pass(b, which, false, dm);
}

mst::LusgsArgs sweep_args(mst_batch* b, int which) {
  mst_ctx* c = b->ctx;
  mst::LusgsArgs la{};
  la.q = qbuf(b, which);
  la.r = c->r;
  la.dq = b->dq;
  la.diag = b->diag;
  la.qn = qbuf(b, 1 - which);
  la.qfn = qfbuf(b, 1 - which);
  la.color = b->color;
  la.c_case = b->c_case;
  la.cfl = b->cfl;
  la.case_tab = b->case_tab;
  la.mu = c->p.mu;
  la.viscous = c->p.viscous;
  la.omega = b->ip.omega;
  la.conv_iter = b->conv_iter;
  la.iter = b->iter;
  la.p_floor = b->ip.p_floor;
  la.case_bad = b->diverged;
  if (b->sweep32) {
    la.qf = qfbuf(b, which);
    la.dqf = b->dqf;
    la.case_tab_f = b->case_tab_f;
    la.mu_f = (float)c->p.mu;
  }
  return la;
}

mst_status enqueue_sweeps(mst_batch* b, int which, int threads) {
  mst_ctx* c = b->ctx;
  mst::LusgsArgs la = sweep_args(b, which);
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = 0; i < b->n_colors; ++i) {
      const int col = pass == 0 ? i : b->n_colors - 1 - i;
      la.col = col;
      const int* cells = b->compact ? b->act_cells : b->color_cells;
      const std::vector<int>& off = b->compact ? b->act_off : b->color_off;
      la.cells = cells + off[col];
      la.n = off[col + 1] - off[col];
      cudaError_t e;
      if (pass == 0)
        e = exact(b) ? mst::exact::lusgs_forward_t(c->dm, la, threads, c->stream)
                     : mst::fast::lusgs_forward_t(c->dm, la, threads, c->stream);
      else
        e = exact(b) ? mst::exact::lusgs_backward_t(c->dm, la, threads, c->stream)
                     : mst::fast::lusgs_backward_t(c->dm, la, threads, c->stream);
      if (e != cudaSuccess)
        return mst_internal_fail(MST_ECUDA, std::string("lusgs sweep: ") + cudaGetErrorString(e));
    }
  }
  return MST_OK;
}

// one implicit iteration from buffer `which` into the other one
mst_status enqueue_iteration(mst_batch* b, int which) {
  mst_status st = enqueue_residual(b, which);
  if (st) return st;
  mst::CaseNormArgs na{};
  na.r = b->ctx->r;
  na.case_first = b->case_first;
  na.first = b->first;
  na.last = b->last;
  na.cfl = b->cfl;
  na.conv_iter = b->conv_iter;
  na.n_conv = b->n_conv;
  na.diverged = b->diverged;
  na.iter = b->iter;
  // the limiter-freezing state machine runs in a case's FP64 phase only
  na.frozen = b->ip.freeze_tol > 0 ? b->frozen : nullptr;
  na.case_lo = b->lo ? b->case_lo : nullptr;
  na.l2_win = b->l2_win;
  na.own_first = b->own_first;
  na.frz_best = b->frz_best;
  na.frz_best_it = b->frz_best_it;
  na.refreeze_window = b->ip.refreeze_window;
  na.restart_it = b->restart_it;
  na.stall_best = b->stall_best;
  na.stall_best_it = b->stall_best_it;
  na.stall_window = b->ip.stall_window;
  na.freeze_tol = b->ip.freeze_tol;
  na.first_fixed = b->first_fixed ? 1 : 0;
  na.part = b->norm_part;
  na.cfl0 = b->ip.cfl0;
  na.cfl_max = b->ip.cfl_max;
  na.tol = b->ip.tol;
  cudaError_t e = exact(b) ? mst::exact::case_norms_t(b->ctx->dm, na, b->n_cases, b->ctx->stream)
                           : mst::fast::case_norms_t(b->ctx->dm, na, b->n_cases, b->ctx->stream);
  if (e != cudaSuccess)
    return mst_internal_fail(MST_ECUDA, std::string("case norms: ") + cudaGetErrorString(e));
  return enqueue_sweeps(b, which, b->threads);
}

// Times the sweeps of the current state for each candidate block size and
// keeps the fastest.  Only the scratch buffers (dq, diag, the other state
// buffer) are written, so the state and the iteration count are untouched.
mst_status autotune(mst_batch* b) {
  mst_ctx* c = b->ctx;
  mst_status st = enqueue_residual(b, b->cur);
  if (st) return st;
  cudaEvent_t e0, e1;
  B_CU(cudaEventCreate(&e0));
  B_CU(cudaEventCreate(&e1));
  float best = 1e30f;
  int pick = 128;
  for (int th : {64, 128, 256}) {
    for (int rep = 0; rep < 2; ++rep) {  // the first repetition warms up
      B_CU(cudaEventRecord(e0, c->stream));
      st = enqueue_sweeps(b, b->cur, th);
      if (st) break;
      B_CU(cudaEventRecord(e1, c->stream));
      B_CU(cudaEventSynchronize(e1));
      float ms = 0.f;
      B_CU(cudaEventElapsedTime(&ms, e0, e1));
      if (rep == 1 && ms < best) {
        best = ms;
        pick = th;
      }
    }
    if (st) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  b->threads = pick;
  return MST_OK;
}

mst_status build_graph(mst_batch* b, int k) {
  mst_ctx* c = b->ctx;
  const int ph = b->lo ? 1 : 0;
  if (b->graph[ph]) {
    cudaGraphExecDestroy(b->graph[ph]);
    b->graph[ph] = nullptr;
  }
  cudaGraph_t g = nullptr;
  B_CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  mst_status st = MST_OK;
  int which = b->cur;
  for (int i = 0; i < k && !st; ++i) {
    st = enqueue_iteration(b, which);
    which = 1 - which;
  }
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess)
    return mst_internal_fail(MST_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->graph[ph], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    return mst_internal_fail(MST_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  b->graph_iters[ph] = k;
  b->graph_cur[ph] = b->cur;
  return MST_OK;
}

CaseProgress progress(mst_batch* b) {
  return CaseProgress{b->cfl,       b->l2_win,        b->stall_best, b->conv_iter,
                      b->diverged,  b->frozen,        b->stall_best_it,
                      b->restart_it, b->n_conv,       b->iter};
}

mst_status reset_progress(mst_batch* b) {
  k_batch_reset<<<(b->n_cases + 255) / 256, 256, 0, b->ctx->stream>>>(
      b->n_cases, b->ip.cfl0, progress(b), nullptr);
  B_CU(cudaGetLastError());
  b->restart_iter.assign(b->n_cases, -1);
  return MST_OK;
}

// Restarts the flagged cases from their fallback states at the current
// iteration: state, per-case progress and (mixed precision) the FP32
// phase start over.  `iters`: the solve loop's iteration count, for the
// phase-switch bookkeeping.
mst_status restart_cases(mst_batch* b, const std::vector<int>& ids, int iters) {
  mst_ctx* c = b->ctx;
  std::vector<int> flag(b->n_cases, 0);
  for (int k : ids) flag[k] = 1;
  int it = 0;
  B_CU(cudaMemcpy(&it, b->iter, sizeof(int), cudaMemcpyDeviceToHost));
  B_CU(cudaMemcpy(b->restart_flag, flag.data(), sizeof(int) * b->n_cases,
                  cudaMemcpyHostToDevice));
  const int nC = c->dm.n_cells;
  k_restart_cells<<<(nC + 255) / 256, 256, 0, c->stream>>>(
      nC, b->c_case, b->restart_flag, b->q_fb, c->q_old, c->q_new, c->qf_old, c->qf_new);
  B_CU(cudaGetLastError());
  k_batch_reset<<<(b->n_cases + 255) / 256, 256, 0, c->stream>>>(
      b->n_cases, b->ip.cfl0, progress(b), b->restart_flag);
  B_CU(cudaGetLastError());
  for (int k : ids) b->restart_iter[k] = it;
  if (b->ip.fp32_until > 0 && c->p.precision == MST_PREC_FP64) {
    // the restarted cases begin in the FP32 phase again
    if (b->lo_h.size() != (size_t)b->n_cases) b->lo_h.assign(b->n_cases, 0);
    if (b->lo_best.size() != (size_t)b->n_cases) {
      b->lo_best.assign(b->n_cases, 1e300);
      b->lo_best_it.assign(b->n_cases, iters);
    }
    for (int k : ids) {
      b->lo_h[k] = 1;
      b->lo_best[k] = 1e300;
      b->lo_best_it[k] = iters;
    }
    B_CU(cudaMemcpy(b->case_lo, b->lo_h.data(), sizeof(int) * b->n_cases,
                    cudaMemcpyHostToDevice));
    b->lo = true;
  }
  B_CU(cudaStreamSynchronize(c->stream));
  return MST_OK;
}

void drop_graphs(mst_batch* b) {
  for (int i = 0; i < 2; ++i)
    if (b->graph[i]) {
      cudaGraphExecDestroy(b->graph[i]);
      b->graph[i] = nullptr;
    }
}

// Lists of the tiles and (per colour) cells of the cases with cv < 0; the
// graphs hold the launches' grids, so they are captured again.
mst_status build_lists(mst_batch* b, const std::vector<int>& cv) {
  mst_ctx* c = b->ctx;
  const int nC = c->dm.n_cells, nT = c->dm.n_tiles;
  std::vector<int> tiles;
  tiles.reserve(nT);
  for (int t = 0; t < nT; ++t) {
    const int k0 = b->c_case_h[t * mst::kTileCells];
    const int k1 = b->c_case_h[std::min((t + 1) * mst::kTileCells, nC) - 1];
    for (int k = k0; k <= k1; ++k)
      if (cv[k] < 0) {
        tiles.push_back(t);
        break;
      }
  }
  std::vector<int> cells;
  cells.reserve(nC);
  b->act_off.assign(b->n_colors + 1, 0);
  for (int col = 0; col < b->n_colors; ++col) {
    for (int i = b->color_off[col]; i < b->color_off[col + 1]; ++i) {
      const int d = b->color_cells_h[i];
      if (cv[b->c_case_h[d]] < 0) cells.push_back(d);
    }
    b->act_off[col + 1] = (int)cells.size();
  }
  if (!tiles.empty())
    B_CU(cudaMemcpy(b->tile_list, tiles.data(), sizeof(int) * tiles.size(),
                    cudaMemcpyHostToDevice));
  if (!cells.empty())
    B_CU(cudaMemcpy(b->act_cells, cells.data(), sizeof(int) * cells.size(),
                    cudaMemcpyHostToDevice));
  c->dm.tile_list = b->tile_list;
  c->dm.n_list = (int)tiles.size();
  b->compact = true;
  b->list_cells = (long long)cells.size();
  drop_graphs(b);
  return MST_OK;
}

// back to launches over every tile and cell
void full_lists(mst_batch* b) {
  if (!b->compact) return;
  b->ctx->dm.tile_list = nullptr;
  b->ctx->dm.n_list = 0;
  b->compact = false;
  b->list_cells = b->ctx->dm.n_cells;
  drop_graphs(b);
}

mst_status run_iterations(mst_batch* b, int n) {
  for (int i = 0; i < n; ++i) {
    mst_status st = enqueue_iteration(b, b->cur);
    if (st) return st;
    b->cur = 1 - b->cur;
  }
  return MST_OK;
}

}  // namespace

extern "C" {

void mst_implicit_params_default(mst_implicit_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->cfl0 = 50.0;
  p->cfl_max = 100.0;
  p->omega = 1.2;
  p->tol = 1e-8;
  p->freeze_tol = 1e-1;
  p->max_iter = 20000;
  p->graph_iters = 20;
  p->autotune = 1;
  p->refreeze_window = 500;
}

mst_status mst_batch_create(const mst_mesh* const* meshes, const mst_case_params* cases,
                            int n_cases, const mst_params* p, const mst_implicit_params* ip,
                            mst_batch** out) {
  if (!meshes || !cases || !p || !ip || !out || n_cases <= 0)
    return mst_internal_fail(MST_EINVAL, "NULL argument or no cases");
  *out = nullptr;
  if (p->reference_quirks)
    return mst_internal_fail(MST_EINVAL, "batches run the corrected scheme (reference_quirks = 0)");
  if (!(ip->cfl0 > 0) || !(ip->cfl_max >= ip->cfl0) || !(ip->omega >= 1.0) || !(ip->tol > 0) ||
      !(ip->freeze_tol >= 0) || !(ip->fp32_until >= 0) ||
      (ip->fp32_until > 0 && p->precision == MST_PREC_FP64_EXACT) ||
      ip->max_iter < 0 || ip->graph_iters < 0 || (ip->graph_iters & 1) ||
      ip->refreeze_window < 0 || ip->stall_window < 0 || ip->restart_after < 0 ||
      ip->restart_projected < 0)
    return mst_internal_fail(MST_EINVAL,
                             "implicit parameters: need cfl0 > 0, cfl_max >= cfl0, omega >= 1, "
                             "tol > 0, max_iter >= 0, graph_iters >= 0 and even, fp32_until >= 0, p_floor >= 0 "
                             "(0 on the exact path), refreeze_window, stall_window, restart_after, "
                             "restart_projected >= 0");
  std::unique_ptr<mst_batch> b(new mst_batch());
  b->ip = *ip;
  b->sweep32 = ip->sweep_fp32 != 0 && p->precision != MST_PREC_FP64_EXACT;
  b->n_cases = n_cases;
  std::vector<const mst::HostMesh*> parts;
  for (int k = 0; k < n_cases; ++k) {
    if (!meshes[k]) return mst_internal_fail(MST_EINVAL, "NULL mesh in the batch");
    parts.push_back(&meshes[k]->host);
  }
  b->mesh = new mst_mesh();
  std::string err;
  int rc = mst::build_union(parts, &b->mesh->host, &err);
  if (rc == mst::kOk) rc = mst::build_layout(b->mesh->host, true, &b->mesh->lay, &err);
  if (rc != mst::kOk) {
    delete b->mesh;
    b->mesh = nullptr;
    return mst_internal_fail(rc == mst::kEMesh ? MST_EMESH : MST_EINVAL, err);
  }
  mst_status st = mst_ctx_create(b->mesh, p, &b->ctx);
  auto cleanup = [&]() {
    if (b->ctx) mst_ctx_destroy(b->ctx);
    for (void* q : b->allocs) cudaFree(q);
    delete b->mesh;
  };
  if (st) {
    cleanup();
    return st;
  }
  const mst::HostMesh& h = b->mesh->host;
  const mst::DevLayout& L = b->mesh->lay;
  const int nC = h.n_cells;
  // greedy colouring in file order (the oracle's om_greedy_colors)
  b->color_file.assign(nC, -1);
  int ncol = 0;
  for (int c = 0; c < nC; ++c) {
    unsigned used = 0;
    for (int k = h.cell_ptr[c]; k < h.cell_ptr[c + 1]; ++k) {
      const int f = h.cell_faces[k];
      if (h.face_cells[2 * f + 1] < 0) continue;
      const int nb = h.cell_nb[k];
      if (nb != c && b->color_file[nb] >= 0 && b->color_file[nb] < 32)
        used |= 1u << b->color_file[nb];
    }
    int pick = 0;
    while (used & (1u << pick)) ++pick;
    b->color_file[c] = pick;
    ncol = std::max(ncol, pick + 1);
  }
  b->n_colors = ncol;
  std::vector<int> color_dev(nC), c_case(nC), case_first(n_cases + 1);
  for (int c = 0; c < nC; ++c) color_dev[L.cell_perm[c]] = b->color_file[c];
  for (int k = 0; k < n_cases; ++k)
    for (int c = h.case_cells[k]; c < h.case_cells[k + 1]; ++c) c_case[L.cell_perm[c]] = k;
  // device cells of case k are contiguous (per-case Morton ranges)
  for (int k = 0; k <= n_cases; ++k) case_first[k] = h.case_cells[k];
  b->color_off.assign(ncol + 1, 0);
  for (int d = 0; d < nC; ++d) b->color_off[color_dev[d] + 1]++;
  for (int i = 0; i < ncol; ++i) b->color_off[i + 1] += b->color_off[i];
  std::vector<int> fill(b->color_off.begin(), b->color_off.end() - 1), cells(nC);
  for (int d = 0; d < nC; ++d) cells[fill[color_dev[d]]++] = d;
  std::vector<double> tab((size_t)mst::kCaseWords * n_cases);
  std::vector<float> tabf(tab.size());
  for (int k = 0; k < n_cases; ++k) {
    const mst_case_params& cp = cases[k];
    const double v[8] = {cp.inlet_q[0], cp.inlet_q[1], cp.inlet_q[2], cp.inlet_q[3],
                         cp.mu, cp.lambda, cp.kappa, cp.cv};
    for (int j = 0; j < 8; ++j) {
      tab[8 * (size_t)k + j] = v[j];
      tabf[8 * (size_t)k + j] = (float)v[j];
    }
  }
  if ((st = bupload(b.get(), &b->color, color_dev)) ||
      (st = bupload(b.get(), &b->color_cells, cells)) ||
      (st = bupload(b.get(), &b->c_case, c_case)) ||
      (st = bupload(b.get(), &b->case_first, case_first)) ||
      (st = bupload(b.get(), &b->case_tab, tab)) ||
      (st = bupload(b.get(), &b->case_tab_f, tabf)) ||
      (st = balloc(b.get(), &b->cfl, sizeof(double) * n_cases)) ||
      (st = balloc(b.get(), &b->first, sizeof(double) * n_cases)) ||
      (st = balloc(b.get(), &b->last, sizeof(double) * n_cases)) ||
      (st = balloc(b.get(), &b->conv_iter, sizeof(int) * n_cases)) ||
      (st = balloc(b.get(), &b->diverged, sizeof(int) * n_cases)) ||
      (st = balloc(b.get(), &b->n_conv, sizeof(int))) ||
      (st = balloc(b.get(), &b->iter, sizeof(int))) ||
      (st = balloc(b.get(), &b->frozen, sizeof(int) * n_cases)) ||
      (st = balloc(b.get(), &b->l2_win, sizeof(double) * n_cases)) ||
      (st = balloc(b.get(), &b->own_first, sizeof(double) * n_cases)) ||
      (st = balloc(b.get(), &b->frz_best, sizeof(double) * n_cases)) ||
      (st = balloc(b.get(), &b->frz_best_it, sizeof(int) * n_cases)) ||
      (st = balloc(b.get(), &b->phi,
                   (size_t)8 * h.n_faces *
                       (p->precision == MST_PREC_FP32 ? sizeof(float) : sizeof(double)))) ||
      (st = balloc(b.get(), &b->dq, sizeof(double4_32a) * (size_t)nC)) ||
      (st = balloc(b.get(), &b->diag, sizeof(double) * (size_t)nC)) ||
      (st = balloc(b.get(), &b->dqf, b->sweep32 ? sizeof(float4) * (size_t)nC : 0)) ||
      (st = balloc(b.get(), &b->norm_part, sizeof(double) * 8 * (size_t)n_cases)) ||
      (st = balloc(b.get(), &b->grad32, p->precision != MST_PREC_FP32 && ip->fp32_until > 0
                                            ? sizeof(float) * 8 * (size_t)nC : 0)) ||
      (st = balloc(b.get(), &b->case_lo, sizeof(int) * n_cases)) ||
      (st = balloc(b.get(), &b->stall_best, sizeof(double) * n_cases)) ||
      (st = balloc(b.get(), &b->stall_best_it, sizeof(int) * n_cases)) ||
      (st = balloc(b.get(), &b->restart_it, sizeof(int) * n_cases)) ||
      (st = balloc(b.get(), &b->restart_flag, sizeof(int) * n_cases)) ||
      (st = balloc(b.get(), &b->tile_list, sizeof(int) * (size_t)L.n_tiles)) ||
      (st = balloc(b.get(), &b->act_cells, sizeof(int) * (size_t)nC)) ||
      (st = reset_progress(b.get()))) {
    cleanup();
    return st;
  }
  // the residual kernels skip the cells of converged cases
  b->ctx->dm.c_case = b->c_case;
  b->ctx->dm.case_conv = b->conv_iter;
  b->c_case_h = std::move(c_case);
  b->color_cells_h = std::move(cells);
  b->list_cells = nC;
  if (cudaStreamSynchronize(b->ctx->stream) != cudaSuccess) {
    cleanup();
    return mst_internal_fail(MST_ECUDA, "batch setup failed");
  }
  *out = b.release();
  return MST_OK;
}

mst_status mst_batch_destroy(mst_batch* b) {
  if (!b) return MST_OK;
  if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
  for (int i = 0; i < 2; ++i)
    if (b->graph[i]) cudaGraphExecDestroy(b->graph[i]);
  for (void* p : b->allocs) cudaFree(p);
  if (b->ctx) mst_ctx_destroy(b->ctx);
  delete b->mesh;
  delete b;
  return MST_OK;
}

mst_status mst_batch_info(const mst_batch* b, mst_batch_info_t* info) {
  if (!b || !info) return mst_internal_fail(MST_EINVAL, "NULL argument");
  info->n_cases = b->n_cases;
  info->n_cells = b->mesh->host.n_cells;
  info->n_faces = b->mesh->host.n_faces;
  info->n_colors = b->n_colors;
  info->sweep_threads = b->threads;
  info->graph_iters = std::max(b->graph_iters[0], b->graph_iters[1]);
  return MST_OK;
}

mst_status mst_batch_colors(const mst_batch* b, int* color) {
  if (!b || !color) return mst_internal_fail(MST_EINVAL, "NULL argument");
  std::memcpy(color, b->color_file.data(), sizeof(int) * b->color_file.size());
  return MST_OK;
}

mst_status mst_batch_set_state(mst_batch* b, const double* q) {
  if (!b || !q) return mst_internal_fail(MST_EINVAL, "NULL argument");
  mst_status st = mst_set_state(b->ctx, q, 4);
  if (st) return st;
  full_lists(b);
  b->cur = 0;
  // a new solve starts in the FP32-residual phase when one is configured
  b->lo = b->ip.fp32_until > 0 && b->ctx->p.precision == MST_PREC_FP64;
  if (b->first_fixed) {
    // graphs captured with caller-set reference L2s: rebuild them
    for (int i = 0; i < 2; ++i)
      if (b->graph[i]) {
        cudaGraphExecDestroy(b->graph[i]);
        b->graph[i] = nullptr;
      }
  }
  b->first_fixed = false;
  b->lo_best.clear();
  b->lo_best_it.clear();
  if (b->lo) {
    b->lo_h.assign(b->n_cases, 1);
    B_CU(cudaMemcpy(b->case_lo, b->lo_h.data(), sizeof(int) * b->n_cases,
                    cudaMemcpyHostToDevice));
  }
  if (b->lo || b->sweep32) {
    cudaError_t e = mst::fast::launch_to_f32(b->ctx->q_old, b->ctx->qf_old, b->ctx->dm.n_cells,
                                             b->ctx->stream);
    if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, cudaGetErrorString(e));
  }
  st = reset_progress(b);
  if (st) return st;
  B_CU(cudaStreamSynchronize(b->ctx->stream));
  return MST_OK;
}

mst_status mst_batch_set_l2_ref(mst_batch* b, const double* l2_ref) {
  if (!b) return mst_internal_fail(MST_EINVAL, "NULL batch");
  if (!l2_ref) {
    b->first_fixed = false;
  } else {
    for (int i = 0; i < b->n_cases; ++i)
      if (!(l2_ref[i] > 0.0))
        return mst_internal_fail(MST_EINVAL, "reference L2 values must be > 0");
    B_CU(cudaMemcpy(b->first, l2_ref, sizeof(double) * b->n_cases, cudaMemcpyHostToDevice));
    b->first_fixed = true;
  }
  // the captured graphs hold the norm arguments: rebuild them
  for (int i = 0; i < 2; ++i)
    if (b->graph[i]) {
      cudaGraphExecDestroy(b->graph[i]);
      b->graph[i] = nullptr;
    }
  return MST_OK;
}

mst_status mst_batch_get_state(mst_batch* b, double* q) {
  if (!b || !q) return mst_internal_fail(MST_EINVAL, "NULL argument");
  mst_ctx* c = b->ctx;
  const int nC = c->dm.n_cells;
  k_batch_gather<<<(nC + 255) / 256, 256, 0, c->stream>>>(qbuf(b, b->cur), c->d.cell_perm,
                                                           c->stage_in, nC);
  B_CU(cudaGetLastError());
  B_CU(cudaMemcpyAsync(q, c->stage_in, sizeof(double4_32a) * (size_t)nC, cudaMemcpyDeviceToHost,
                       c->stream));
  B_CU(cudaStreamSynchronize(c->stream));
  return MST_OK;
}

mst_status mst_batch_iterate(mst_batch* b, int n) {
  if (!b || n < 0) return mst_internal_fail(MST_EINVAL, "bad argument");
  mst_status st = run_iterations(b, n);
  if (st) return st;
  B_CU(cudaStreamSynchronize(b->ctx->stream));
  return MST_OK;
}

mst_status mst_batch_solve(mst_batch* b, mst_batch_result* res) {
  if (!b) return mst_internal_fail(MST_EINVAL, "NULL batch");
  mst_ctx* c = b->ctx;
  mst_status st;
  if (b->ip.autotune && !b->tuned) {
    st = autotune(b);
    if (st) return st;
    b->tuned = true;
  }
  const int k = b->ip.graph_iters;
  auto ensure_graph = [&]() -> mst_status {
    const int ph = b->lo ? 1 : 0;
    if (k > 0 && (b->graph_iters[ph] != k || b->graph_cur[ph] != b->cur || !b->graph[ph])) {
      // the kernels' one-time attribute setup runs before capture
      mst_status s2 = enqueue_residual(b, b->cur);
      if (s2) return s2;
      B_CU(cudaStreamSynchronize(c->stream));
      return build_graph(b, k);
    }
    return MST_OK;
  };
  st = ensure_graph();
  if (st) return st;
  int h[2] = {0, 0};
  B_CU(cudaMemcpy(&h[0], b->iter, sizeof(int), cudaMemcpyDeviceToHost));
  const int start = h[0];
  B_CU(cudaEventRecord(c->ev0, c->stream));
  int done = 0, iters = 0, last_done = 0;
  // restart_projected: per case the L2 at the start of the current window
  const int pw = b->ip.restart_projected;
  std::vector<double> proj_l2(b->n_cases, -1.0);
  std::vector<int> proj_slow(b->n_cases, 0);
  int next_proj = pw > 0 ? pw : 0;
  std::vector<double> f(b->n_cases), l(b->n_cases);
  std::vector<int> cv(b->n_cases), dv(b->n_cases);
  const std::vector<int>& case_cells = b->mesh->host.case_cells;
  while (iters < b->ip.max_iter) {
    if (k > 0 && iters + k <= b->ip.max_iter) {
      B_CU(cudaGraphLaunch(b->graph[b->lo ? 1 : 0], c->stream));
      iters += k;  // k is even: the state is back in the same buffer
    } else {
      st = run_iterations(b, 1);
      if (st) return st;
      iters += 1;
    }
    B_CU(cudaMemcpyAsync(&h[1], b->n_conv, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    B_CU(cudaStreamSynchronize(c->stream));
    done = h[1];
    bool restarted = false;
    const int now = start + iters;  // iterations since the state was set
    const bool stall = b->ip.stall_window > 0 && done > 0;
    const bool late = b->ip.restart_after > 0 && now >= b->ip.restart_after;
    const bool proj = pw > 0 && now >= next_proj;
    if (b->has_fb && (stall || late || proj)) {
      // a case retired as stalled, not converged restart_after iterations
      // after the state was set, or projected past max_iter restarts from
      // its fallback state, once
      B_CU(cudaMemcpy(dv.data(), b->diverged, sizeof(int) * dv.size(), cudaMemcpyDeviceToHost));
      B_CU(cudaMemcpy(cv.data(), b->conv_iter, sizeof(int) * cv.size(), cudaMemcpyDeviceToHost));
      std::vector<char> slow(b->n_cases, 0);
      if (proj) {
        B_CU(cudaMemcpy(f.data(), b->first, sizeof(double) * f.size(), cudaMemcpyDeviceToHost));
        B_CU(cudaMemcpy(l.data(), b->last, sizeof(double) * l.size(), cudaMemcpyDeviceToHost));
        for (int i = 0; i < b->n_cases; ++i) {
          if (b->lo && b->lo_h[i]) {
            // the FP32 phase levels off by design: the window starts
            // when the case leaves it
            proj_l2[i] = -1.0;
            continue;
          }
          if (cv[i] < 0 && b->restart_iter[i] < 0 && proj_l2[i] > 0.0 && l[i] > 0.0 &&
              f[i] > 0.0) {
            // iterations still needed at the last window's rate (decades
            // per iteration); no progress projects to infinity.  Two
            // windows in a row (a plateau before the limiter freezes is
            // not a slow case)
            const double rate = std::log10(proj_l2[i] / l[i]) / pw;
            const double need = std::log10(l[i] / (b->ip.tol * f[i]));
            const bool past =
                need > 0.0 && (rate <= 0.0 || now + need / rate > (double)b->ip.max_iter);
            proj_slow[i] = past ? proj_slow[i] + 1 : 0;
            slow[i] = proj_slow[i] >= 2;
          }
          proj_l2[i] = l[i];
        }
        next_proj = now + pw;
      }
      std::vector<int> ids;
      for (int i = 0; i < b->n_cases; ++i)
        if (b->restart_iter[i] < 0 &&
            ((stall && dv[i] == 2) || (late && cv[i] < 0) || (slow[i] && cv[i] < 0)))
          ids.push_back(i);
      if (!ids.empty()) {
        st = restart_cases(b, ids, iters);
        if (st) return st;
        for (int i : ids) {
          done -= cv[i] >= 0;  // retired cases count again
          cv[i] = -1;
        }
        restarted = true;
        st = ensure_graph();
        if (st) return st;
      }
    }
    if (done >= b->n_cases) break;
    if (done != last_done || restarted) {
      // compaction: once the unconverged cases hold at most 3/4 of the
      // cells the launches cover, the lists shrink to theirs (a restarted
      // case must be in them again)
      if (!restarted)
        B_CU(cudaMemcpy(cv.data(), b->conv_iter, sizeof(int) * cv.size(), cudaMemcpyDeviceToHost));
      long long act = 0;
      for (int i = 0; i < b->n_cases; ++i)
        if (cv[i] < 0) act += case_cells[i + 1] - case_cells[i];
      if ((restarted && b->compact) || 4 * act <= 3 * b->list_cells) {
        st = build_lists(b, cv);
        if (st) return st;
        st = ensure_graph();
        if (st) return st;
      }
      last_done = done;
    }
    if (b->lo) {
      // a case leaves the FP32 phase once converged, below fp32_until, or
      // stagnating in FP32 (its L2 has not fallen by 10% for win
      // iterations: the FP32 residual's floor); each case on its own
      B_CU(cudaMemcpy(f.data(), b->first, sizeof(double) * f.size(), cudaMemcpyDeviceToHost));
      B_CU(cudaMemcpy(l.data(), b->last, sizeof(double) * l.size(), cudaMemcpyDeviceToHost));
      B_CU(cudaMemcpy(cv.data(), b->conv_iter, sizeof(int) * cv.size(), cudaMemcpyDeviceToHost));
      if (b->lo_best.size() != (size_t)b->n_cases) {
        b->lo_best.assign(b->n_cases, 1e300);
        b->lo_best_it.assign(b->n_cases, iters);
      }
      const int win = b->ip.fp32_window > 0 ? b->ip.fp32_window : 500;
      int left = 0;
      bool moved = false;
      for (int i = 0; i < b->n_cases; ++i) {
        if (!b->lo_h[i]) continue;
        bool ready = cv[i] >= 0 || l[i] <= b->ip.fp32_until * f[i];
        if (!ready) {
          if (l[i] < 0.9 * b->lo_best[i]) {
            b->lo_best[i] = l[i];
            b->lo_best_it[i] = iters;
          }
          ready = iters - b->lo_best_it[i] >= win;
        }
        if (ready) {
          b->lo_h[i] = 0;
          moved = true;
        } else {
          ++left;
        }
      }
      if (left == 0) {
        // every case in FP64: the single-phase iterations from here on
        b->lo = false;
        st = ensure_graph();
        if (st) return st;
      } else if (moved) {
        // read by the next iterations' launches (same stream)
        B_CU(cudaMemcpy(b->case_lo, b->lo_h.data(), sizeof(int) * b->n_cases,
                        cudaMemcpyHostToDevice));
      }
    }
  }
  B_CU(cudaEventRecord(c->ev1, c->stream));
  B_CU(cudaEventSynchronize(c->ev1));
  float ms = 0.f;
  B_CU(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  if (res) {
    B_CU(cudaMemcpy(dv.data(), b->diverged, sizeof(int) * dv.size(), cudaMemcpyDeviceToHost));
    int n_div = 0, n_stall = 0, n_rs = 0;
    for (int x : dv) {
      n_div += x == 1;
      n_stall += x == 2;
    }
    for (int x : b->restart_iter) n_rs += x >= 0;
    res->iterations = iters;
    res->total_iterations = start + iters;
    res->n_converged = done - n_div - n_stall;
    res->ms = ms;
    res->n_diverged = n_div;
    res->n_stalled = n_stall;
    res->n_restarted = n_rs;
  }
  return MST_OK;
}

mst_status mst_batch_case_status(mst_batch* b, int* conv_iter, double* first_l2,
                                 double* last_l2) {
  if (!b) return mst_internal_fail(MST_EINVAL, "NULL batch");
  const size_t n = (size_t)b->n_cases;
  if (conv_iter) {
    std::vector<int> dv(n);
    B_CU(cudaMemcpy(conv_iter, b->conv_iter, sizeof(int) * n, cudaMemcpyDeviceToHost));
    B_CU(cudaMemcpy(dv.data(), b->diverged, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i)
      if (dv[i]) conv_iter[i] = dv[i] == 2 ? MST_CASE_STALLED : MST_CASE_DIVERGED;
  }
  if (first_l2) B_CU(cudaMemcpy(first_l2, b->first, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (last_l2) B_CU(cudaMemcpy(last_l2, b->last, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return MST_OK;
}

mst_status mst_batch_set_fallback(mst_batch* b, const double* q) {
  if (!b) return mst_internal_fail(MST_EINVAL, "NULL batch");
  if (!q) {
    b->has_fb = false;
    return MST_OK;
  }
  mst_ctx* c = b->ctx;
  const int nC = c->dm.n_cells;
  mst_status st = MST_OK;
  if (!b->q_fb && (st = balloc(b, &b->q_fb, sizeof(double4_32a) * (size_t)nC))) return st;
  // host rows (file order) -> device order, through the context's staging
  B_CU(cudaMemcpyAsync(c->stage_in, q, sizeof(double4_32a) * (size_t)nC, cudaMemcpyHostToDevice,
                       c->stream));
  k_batch_gather<<<(nC + 255) / 256, 256, 0, c->stream>>>(c->stage_in, c->d.cell_iperm, b->q_fb,
                                                           nC);
  B_CU(cudaGetLastError());
  B_CU(cudaStreamSynchronize(c->stream));
  b->has_fb = true;
  return MST_OK;
}

mst_status mst_batch_restart(mst_batch* b, const int* cases, int n) {
  if (!b || (n > 0 && !cases) || n < 0) return mst_internal_fail(MST_EINVAL, "bad argument");
  if (!b->has_fb) return mst_internal_fail(MST_EINVAL, "no fallback states (mst_batch_set_fallback)");
  std::vector<int> ids(cases, cases + n);
  std::vector<char> seen(b->n_cases, 0);
  for (int k : ids) {
    if (k < 0 || k >= b->n_cases || seen[k])
      return mst_internal_fail(MST_EINVAL, "case index out of range or repeated");
    seen[k] = 1;
  }
  if (ids.empty()) return MST_OK;
  // launches over every tile again (the solve compacts them anew)
  full_lists(b);
  return restart_cases(b, ids, 0);
}

mst_status mst_batch_case_restarts(mst_batch* b, int* restart_iter) {
  if (!b || !restart_iter) return mst_internal_fail(MST_EINVAL, "NULL argument");
  std::memcpy(restart_iter, b->restart_iter.data(), sizeof(int) * b->n_cases);
  return MST_OK;
}

}  // extern "C"
