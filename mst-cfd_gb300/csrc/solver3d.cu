// The 3D residual path behind the C ABI (mst_ctx3d_*, include/mstcfd.h):
// device layout upload, RK2 stepping with the state resident in HBM, the
// residual and gradient for parity checks, the kinetic-energy diagnostic,
// and per-kernel event timing.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ctx.hpp"
#include "devtypes3d.hpp"
#include "launch3d.hpp"
#include "mesh3d.hpp"

namespace {

mst_status fail3(mst_status s, const std::string& msg) { return mst_internal_fail(s, msg); }

#define C3(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail3(MST_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
  } while (0)

}  // namespace

struct mst_ctx3d {
  mst_params3d p{};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  mst::DevMesh3 dm{};
  std::vector<int> cell_perm;  // file -> device
  int n_cell_faces = 0, n_borrowed = 0;
  std::vector<void*> allocs;
  size_t bytes = 0;
  // FP64 state buffers (cur, stage, next) or float pairs for the FP32 path
  double* q[3] = {};
  float4 *h4[3] = {}, *l4[3] = {};
  float *h1[3] = {}, *l1[3] = {};
  double* qtmp = nullptr;  // [nC][5] conversions / residual
  void* grad = nullptr;
  double* dt_part = nullptr;
  double* scal = nullptr;  // [0] dt, [1] time
  float* dt_ff = nullptr;
  double* ke_part = nullptr;
  double* ke_out = nullptr;
  int cur = 0;
  int last_launches = 0;
  double last_ms = 0.0;
  // per-kernel event timing
  bool profiling = false;
  struct Pending {
    int k;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  std::vector<std::string> kname;
  std::vector<int> klaunch;
  std::vector<double> kms;
};

namespace {

bool exact3(const mst_ctx3d* c) { return c->p.precision == MST_PREC_FP64_EXACT; }
bool f32(const mst_ctx3d* c) { return c->p.precision == MST_PREC_FP32; }

template <class T>
mst_status alloc3(mst_ctx3d* c, T** p, size_t count) {
  void* v = nullptr;
  const size_t b = std::max<size_t>(count, 1) * sizeof(T);
  C3(cudaMalloc(&v, b));
  c->allocs.push_back(v);
  c->bytes += b;
  *p = static_cast<T*>(v);
  return MST_OK;
}

template <class T, class S>
mst_status upload3(mst_ctx3d* c, const T** dst, const std::vector<S>& src) {
  T* d = nullptr;
  mst_status st = alloc3(c, &d, src.size());
  if (st) return st;
  std::vector<T> tmp(src.begin(), src.end());
  if (!tmp.empty()) C3(cudaMemcpy(d, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice));
  *dst = d;
  return MST_OK;
}

cudaEvent_t take_ev(mst_ctx3d* c) {
  if (!c->pool.empty()) {
    cudaEvent_t e = c->pool.back();
    c->pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

struct Prof3 {
  mst_ctx3d* c;
  int k = -1;
  cudaEvent_t a = nullptr, b = nullptr;
  Prof3(mst_ctx3d* ctx, const char* name) : c(ctx) {
    if (!c->profiling) return;
    for (size_t i = 0; i < c->kname.size() && k < 0; ++i)
      if (c->kname[i] == name) k = (int)i;
    if (k < 0) {
      c->kname.push_back(name);
      c->klaunch.push_back(0);
      c->kms.push_back(0.0);
      k = (int)c->kname.size() - 1;
    }
    a = take_ev(c);
    b = take_ev(c);
    cudaEventRecord(a, c->stream);
  }
  ~Prof3() {
    if (k < 0) return;
    cudaEventRecord(b, c->stream);
    c->pending.push_back({k, a, b});
  }
};

void drain3(mst_ctx3d* c) {
  if (c->pending.empty()) return;
  cudaStreamSynchronize(c->stream);
  for (auto& p : c->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      c->klaunch[p.k] += 1;
      c->kms[p.k] += ms;
    }
    c->pool.push_back(p.a);
    c->pool.push_back(p.b);
  }
  c->pending.clear();
}

// stage arguments on buffer set `in` (and `prev` for the second RK stage)
mst::Step3Args args3(mst_ctx3d* c, int in, int out, int prev, int stage) {
  mst::Step3Args a{};
  a.q = c->q[in];
  a.qn = out >= 0 ? c->q[out] : nullptr;
  a.q0 = prev >= 0 ? c->q[prev] : nullptr;
  a.h4 = c->h4[in];
  a.h1 = c->h1[in];
  a.l4 = c->l4[in];
  a.l1 = c->l1[in];
  if (out >= 0) {
    a.nh4 = c->h4[out];
    a.nh1 = c->h1[out];
    a.nl4 = c->l4[out];
    a.nl1 = c->l1[out];
  }
  if (prev >= 0) {
    a.ph4 = c->h4[prev];
    a.ph1 = c->h1[prev];
    a.pl4 = c->l4[prev];
    a.pl1 = c->l1[prev];
  }
  a.grad = c->grad;
  a.scal = c->scal;
  a.dt_ff = c->dt_ff;
  a.stage = stage;
  a.limiter = c->p.limiter;
  a.mu = c->p.mu;
  a.lam = c->p.lambda;
  a.kappa = c->p.kappa;
  a.cv = c->p.cv;
  a.mu_f = (float)c->p.mu;
  a.lam_f = (float)c->p.lambda;
  a.kappa_f = (float)c->p.kappa;
  a.cv_f = (float)c->p.cv;
  for (int k = 0; k < 5; ++k) {
    a.inlet[k] = c->p.inlet_q[k];
    a.inlet_f[k] = (float)c->p.inlet_q[k];
  }
  return a;
}

cudaError_t grad3(mst_ctx3d* c, const mst::Step3Args& a, double* dt_part) {
  Prof3 pr(c, "k3_gradient");
  ++c->last_launches;
  return exact3(c) ? mst::exact3::gradient(c->p.precision, c->dm, a, c->grad, c->p.cfl, dt_part,
                                           c->stream)
                   : mst::fast3::gradient(c->p.precision, c->dm, a, c->grad, c->p.cfl, dt_part,
                                          c->stream);
}

cudaError_t flux3(mst_ctx3d* c, const mst::Step3Args& a, int mode) {
  Prof3 pr(c, "k3_flux_update");
  ++c->last_launches;
  return exact3(c) ? mst::exact3::flux_update(c->p.precision, c->p.order, c->p.viscous != 0,
                                              mode, c->dm, a, c->stream)
                   : mst::fast3::flux_update(c->p.precision, c->p.order, c->p.viscous != 0,
                                             mode, c->dm, a, c->stream);
}

// the residual of the current state into c->qtmp (device order)
mst_status residual_dev(mst_ctx3d* c) {
  mst::Step3Args a = args3(c, c->cur, -1, -1, 0);
  a.r_out = c->qtmp;
  if (c->p.order == 2) C3(grad3(c, a, nullptr));
  C3(flux3(c, a, 3));
  return MST_OK;
}

mst_status to_file_order(mst_ctx3d* c, const double* dev, int width, double* out) {
  const int nC = c->dm.n_cells;
  std::vector<double> h((size_t)nC * width);
  C3(cudaStreamSynchronize(c->stream));
  C3(cudaMemcpy(h.data(), dev, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int f = 0; f < nC; ++f)
    std::memcpy(out + (size_t)f * width, h.data() + (size_t)c->cell_perm[f] * width,
                sizeof(double) * width);
  return MST_OK;
}

}  // namespace

extern "C" {

mst_status mst_mesh3d_from_arrays(int n_nodes, const double* node_xyz, int n_cells, int n_faces,
                                  const int* face_ptr, const int* face_nodes,
                                  const int* face_cells, int n_zones, const int* zones,
                                  const double* c1_shift, mst_mesh3d** out) {
  if (!out || !node_xyz || !face_ptr || !face_nodes || !face_cells || !zones || n_nodes <= 0 ||
      n_cells <= 0 || n_faces <= 0 || n_zones <= 0)
    return fail3(MST_EINVAL, "mst_mesh3d_from_arrays: NULL or empty argument");
  *out = nullptr;
  std::unique_ptr<mst_mesh3d> m(new mst_mesh3d());
  mst::HostMesh3D& h = m->host;
  h.n_nodes = n_nodes;
  h.n_cells = n_cells;
  h.n_faces = n_faces;
  h.node_xyz.assign(node_xyz, node_xyz + 3 * (size_t)n_nodes);
  h.face_ptr.assign(face_ptr, face_ptr + n_faces + 1);
  if (h.face_ptr[0] != 0)
    return fail3(MST_EINVAL, "mst_mesh3d_from_arrays: face_ptr must start at 0");
  for (int f = 0; f < n_faces; ++f) {
    const int k = h.face_ptr[f + 1] - h.face_ptr[f];
    if (k != 3 && k != 4)
      return fail3(MST_EMESH, "mst_mesh3d_from_arrays: faces need 3 or 4 nodes");
  }
  h.face_nodes.assign(face_nodes, face_nodes + h.face_ptr[n_faces]);
  for (int nd : h.face_nodes)
    if (nd < 0 || nd >= n_nodes)
      return fail3(MST_EMESH, "mst_mesh3d_from_arrays: node id out of range");
  h.face_cells.assign(face_cells, face_cells + 2 * (size_t)n_faces);
  h.face_type.assign(n_faces, 0);
  for (int z = 0; z < n_zones; ++z) {
    const int first = zones[4 * z + 1], last = zones[4 * z + 2], ty = zones[4 * z + 3];
    if (first < 1 || last > n_faces || first > last + 1)
      return fail3(MST_EMESH, "mst_mesh3d_from_arrays: bad zone range");
    h.zone.insert(h.zone.end(), {zones[4 * z], first, last, ty});
    for (int f = first - 1; f < last; ++f) h.face_type[f] = ty;
    if (ty == mst::kInterior) h.n_int_faces = std::max(h.n_int_faces, last);
  }
  if (c1_shift) m->c1_shift.assign(c1_shift, c1_shift + 3 * (size_t)n_faces);
  m->from_arrays = true;
  *out = m.release();
  return MST_OK;
}

void mst_params3d_default(mst_params3d* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->precision = MST_PREC_FP32;
  p->order = 2;
  p->limiter = MST_LIMITER_VANALBADA;
  p->cv = 1.0 / (1.4 * 0.4);
  p->inlet_q[0] = 1.0;
  p->inlet_q[4] = 1.0 / (1.4 * 0.4);
  p->cfl = 0.5;
}

mst_status mst_ctx3d_create(const mst_mesh3d* mesh, const mst_params3d* p, mst_ctx3d** out) {
  if (!mesh || !p || !out) return fail3(MST_EINVAL, "NULL argument");
  *out = nullptr;
  if (p->precision < MST_PREC_FP64_EXACT || p->precision > MST_PREC_FP32)
    return fail3(MST_EINVAL, "unknown precision");
  if (p->order != 1 && p->order != 2) return fail3(MST_EINVAL, "order must be 1 or 2");
  if (p->limiter < MST_LIMITER_NONE || p->limiter > MST_LIMITER_VANALBADA)
    return fail3(MST_EINVAL, "unknown limiter");
  if (p->viscous && p->order != 2)
    return fail3(MST_EINVAL, "the viscous term needs order 2 (cell gradients)");
  if (p->viscous && !(p->mu >= 0 && p->kappa >= 0 && p->cv > 0))
    return fail3(MST_EINVAL, "bad viscous coefficients");
  if (!(p->cfl > 0)) return fail3(MST_EINVAL, "cfl must be > 0");
  mst::SolverMesh3D sm;
  mst::DevLayout3D L;
  std::string err;
  int rc = mst::build_solver3d(mesh->host, mesh->c1_shift, &sm, &err);
  if (rc == mst::kOk) rc = mst::build_layout3d(sm, &L, &err);
  if (rc != mst::kOk) return fail3(rc == mst::kEMesh ? MST_EMESH : MST_EINVAL, err);
  std::unique_ptr<mst_ctx3d> c(new mst_ctx3d());
  c->p = *p;
  if (!f32(c.get()) && p->order == 2 &&
      sizeof(double) * 18 * (size_t)L.max_tile_faces > 200 * 1024)
    return fail3(MST_EMESH, "a cell tile touches too many faces for shared memory");
  auto cleanup = [&]() {
    for (void* v : c->allocs) cudaFree(v);
    if (c->stream) cudaStreamDestroy(c->stream);
  };
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    cleanup();
    return fail3(MST_ECUDA, "stream/event creation failed");
  }
  const int nC = L.n_cells, nF = L.n_faces, tot = L.c_ptr[nC];
  mst::DevMesh3& d = c->dm;
  d.n_cells = nC;
  d.n_faces = nF;
  d.n_tiles = L.n_tiles;
  d.max_tile_faces = std::max(L.max_tile_faces, 1);
  std::vector<int2> c0c1(nF);
  for (int f = 0; f < nF; ++f) c0c1[f] = make_int2(L.f_c0c1[2 * (size_t)f], L.f_c0c1[2 * (size_t)f + 1]);
  std::vector<double> ivol(nC);
  std::vector<float2> ivff(nC);
  for (int i = 0; i < nC; ++i) {
    ivol[i] = 1.0 / L.c_vol[i];
    const float hi = (float)ivol[i];
    ivff[i] = make_float2(hi, (float)(ivol[i] - (double)hi));
  }
  // packed FP32 copies of the geometry
  std::vector<float4> fde(nF), fr0(nF), fr1(nF), cdw(tot);
  std::vector<float> cw1(tot);
  for (int f = 0; f < nF; ++f) {
    const double* dv = &L.f_dir[3 * (size_t)f];
    const double* a0 = &L.f_r0[3 * (size_t)f];
    const double* a1 = &L.f_r1[3 * (size_t)f];
    fde[f] = make_float4((float)dv[0], (float)dv[1], (float)dv[2], (float)L.f_eta[f]);
    fr0[f] = make_float4((float)a0[0], (float)a0[1], (float)a0[2], 0.0f);
    fr1[f] = make_float4((float)a1[0], (float)a1[1], (float)a1[2], 0.0f);
  }
  for (int k = 0; k < tot; ++k) {
    const double* dv = &L.cf_dir[3 * (size_t)k];
    cdw[k] = make_float4((float)dv[0], (float)dv[1], (float)dv[2], (float)L.cf_w[2 * (size_t)k]);
    cw1[k] = (float)L.cf_w[2 * (size_t)k + 1];
  }
  mst_status st = MST_OK;
  if ((st = upload3(c.get(), &d.f_c0c1, c0c1)) || (st = upload3(c.get(), &d.f_info, L.f_info)) ||
      (st = upload3(c.get(), &d.f_dir, L.f_dir)) || (st = upload3(c.get(), &d.f_r0, L.f_r0)) ||
      (st = upload3(c.get(), &d.f_r1, L.f_r1)) || (st = upload3(c.get(), &d.f_eta, L.f_eta)) ||
      (st = upload3(c.get(), &d.f_dir_eta32, fde)) ||
      (st = upload3(c.get(), &d.f_r0_32, fr0)) || (st = upload3(c.get(), &d.f_r1_32, fr1)) ||
      (st = upload3(c.get(), &d.c_vol, L.c_vol)) ||
      (st = upload3(c.get(), &d.c_ivol, ivol)) || (st = upload3(c.get(), &d.c_ivol_ff, ivff)) ||
      (st = upload3(c.get(), &d.c_ptr, L.c_ptr)) ||
      (st = upload3(c.get(), &d.cf_slot, L.cf_slot)) ||
      (st = upload3(c.get(), &d.cf_nb, L.cf_nb)) || (st = upload3(c.get(), &d.cf_w, L.cf_w)) ||
      (st = upload3(c.get(), &d.cf_dir, L.cf_dir)) ||
      (st = upload3(c.get(), &d.cf_dw32, cdw)) || (st = upload3(c.get(), &d.cf_w1_32, cw1)) ||
      (st = upload3(c.get(), &d.t_own_ptr, L.t_own_ptr)) ||
      (st = upload3(c.get(), &d.t_bor_ptr, L.t_bor_ptr)) ||
      (st = upload3(c.get(), &d.t_bor, L.t_bor))) {
    cleanup();
    return st;
  }
  const int nb = (nC + 255) / 256;
  const bool pairs = f32(c.get());
  for (int i = 0; i < 3 && !st; ++i) {
    if (pairs) {
      (st = alloc3(c.get(), &c->h4[i], nC)) || (st = alloc3(c.get(), &c->h1[i], nC)) ||
          (st = alloc3(c.get(), &c->l4[i], nC)) || (st = alloc3(c.get(), &c->l1[i], nC));
    } else {
      st = alloc3(c.get(), &c->q[i], 5 * (size_t)nC);
    }
  }
  if (st || (st = alloc3(c.get(), &c->qtmp, 5 * (size_t)nC)) ||
      (st = alloc3(c.get(), (char**)&c->grad,
                   mst::kGrad3 * (size_t)nC * (pairs ? sizeof(float) : sizeof(double)))) ||
      (st = alloc3(c.get(), &c->dt_part, nb)) || (st = alloc3(c.get(), &c->scal, 2)) ||
      (st = alloc3(c.get(), &c->dt_ff, 2)) || (st = alloc3(c.get(), &c->ke_part, 2 * (size_t)nb)) ||
      (st = alloc3(c.get(), &c->ke_out, 2))) {
    cleanup();
    return st;
  }
  if (cudaMemset(c->scal, 0, 2 * sizeof(double)) != cudaSuccess) {
    cleanup();
    return fail3(MST_ECUDA, "memset failed");
  }
  c->cell_perm = L.cell_perm;
  c->n_cell_faces = tot;
  c->n_borrowed = (int)L.t_bor.size();
  *out = c.release();
  return MST_OK;
}

mst_status mst_ctx3d_destroy(mst_ctx3d* c) {
  if (!c) return MST_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (void* v : c->allocs) cudaFree(v);
  for (auto& p : c->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : c->pool) cudaEventDestroy(e);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return MST_OK;
}

mst_status mst_ctx3d_info_get(mst_ctx3d* c, mst_ctx3d_info* info) {
  if (!c || !info) return fail3(MST_EINVAL, "NULL argument");
  info->n_cells = c->dm.n_cells;
  info->n_faces = c->dm.n_faces;
  info->n_tiles = c->dm.n_tiles;
  info->max_tile_faces = c->dm.max_tile_faces;
  info->n_cell_faces = c->n_cell_faces;
  info->n_borrowed = c->n_borrowed;
  info->device_bytes = c->bytes;
  return MST_OK;
}

mst_status mst_ctx3d_set_state(mst_ctx3d* c, const double* q) {
  if (!c || !q) return fail3(MST_EINVAL, "NULL argument");
  const int nC = c->dm.n_cells;
  std::vector<double> h(5 * (size_t)nC);
  for (int f = 0; f < nC; ++f)
    std::memcpy(h.data() + 5 * (size_t)c->cell_perm[f], q + 5 * (size_t)f, 5 * sizeof(double));
  double* dst = f32(c) ? c->qtmp : c->q[c->cur];
  C3(cudaMemcpyAsync(dst, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice,
                     c->stream));
  if (f32(c)) {
    const int i = c->cur;
    C3(mst::fast3::pairs(true, c->qtmp, nC, c->h4[i], c->h1[i], c->l4[i], c->l1[i], c->stream));
  }
  C3(cudaStreamSynchronize(c->stream));
  return MST_OK;
}

mst_status mst_ctx3d_get_state(mst_ctx3d* c, double* q) {
  if (!c || !q) return fail3(MST_EINVAL, "NULL argument");
  const double* src = c->q[c->cur];
  if (f32(c)) {
    const int i = c->cur;
    C3(mst::fast3::pairs(false, c->qtmp, c->dm.n_cells, c->h4[i], c->h1[i], c->l4[i], c->l1[i],
                         c->stream));
    src = c->qtmp;
  }
  return to_file_order(c, src, 5, q);
}

mst_status mst_ctx3d_residual(mst_ctx3d* c, double* r) {
  if (!c || !r) return fail3(MST_EINVAL, "NULL argument");
  mst_status st = residual_dev(c);
  if (st) return st;
  return to_file_order(c, c->qtmp, 5, r);
}

mst_status mst_ctx3d_gradient(mst_ctx3d* c, double* g) {
  if (!c || !g) return fail3(MST_EINVAL, "NULL argument");
  if (c->p.order != 2) return fail3(MST_EINVAL, "gradients exist for order 2 only");
  mst::Step3Args a = args3(c, c->cur, -1, -1, 0);
  C3(grad3(c, a, nullptr));
  const int nC = c->dm.n_cells;
  const int W = mst::kGrad3;
  std::vector<double> gd(W * (size_t)nC);
  C3(cudaStreamSynchronize(c->stream));
  if (f32(c)) {
    std::vector<float> gf(gd.size());
    C3(cudaMemcpy(gf.data(), c->grad, gf.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < gd.size(); ++i) gd[i] = gf[i];
  } else {
    C3(cudaMemcpy(gd.data(), c->grad, gd.size() * sizeof(double), cudaMemcpyDeviceToHost));
  }
  for (int f = 0; f < nC; ++f)
    std::memcpy(g + 15 * (size_t)f, gd.data() + W * (size_t)c->cell_perm[f], 15 * sizeof(double));
  return MST_OK;
}

mst_status mst_ctx3d_step(mst_ctx3d* c, int nsteps, double t_end, double* time) {
  if (!c || nsteps < 0) return fail3(MST_EINVAL, "bad arguments");
  c->last_launches = 0;
  const int nb = (c->dm.n_cells + 255) / 256;
  C3(cudaEventRecord(c->ev0, c->stream));
  for (int s = 0; s < nsteps; ++s) {
    const int in = c->cur, stg = (c->cur + 1) % 3, nxt = (c->cur + 2) % 3;
    mst::Step3Args a0 = args3(c, in, stg, -1, 0);
    C3(grad3(c, a0, c->dt_part));
    {
      Prof3 pr(c, "k3_finalize_dt");
      ++c->last_launches;
      C3(mst::fast3::finalize_dt(c->dt_part, nb, t_end, c->scal, c->dt_ff, c->stream));
    }
    C3(flux3(c, a0, f32(c) ? 1 : 0));
    mst::Step3Args a1 = args3(c, stg, nxt, in, 1);
    if (c->p.order == 2) C3(grad3(c, a1, nullptr));
    C3(flux3(c, a1, f32(c) ? 1 : 0));
    c->cur = nxt;
  }
  C3(cudaEventRecord(c->ev1, c->stream));
  C3(cudaEventSynchronize(c->ev1));
  float ms = 0.f;
  C3(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last_ms = ms;
  drain3(c);
  double sc[2] = {0.0, 0.0};
  C3(cudaMemcpy(sc, c->scal, sizeof sc, cudaMemcpyDeviceToHost));
  if (time) *time = sc[1];
  // a step of zero length before t_end: the CFL step of some cell was not
  // positive (NaN, non-positive density or pressure)
  if (nsteps > 0 && !(sc[0] > 0.0) && !(t_end > 0.0 && sc[1] >= t_end))
    return fail3(MST_EDIVERGED, "mst_ctx3d_step: non-positive CFL step (NaN or non-positive "
                                "density or pressure)");
  return MST_OK;
}

mst_status mst_ctx3d_last_timing(mst_ctx3d* c, double* ms, int* launches) {
  if (!c) return fail3(MST_EINVAL, "NULL context");
  if (ms) *ms = c->last_ms;
  if (launches) *launches = c->last_launches;
  return MST_OK;
}

mst_status mst_ctx3d_kinetic_energy(mst_ctx3d* c, double* ke, double* vol) {
  if (!c) return fail3(MST_EINVAL, "NULL context");
  mst::Step3Args a = args3(c, c->cur, -1, -1, 0);
  C3((exact3(c) ? mst::exact3::kinetic : mst::fast3::kinetic)(c->p.precision, c->dm, a,
                                                               c->ke_part, c->ke_out, c->stream));
  double h[2];
  C3(cudaStreamSynchronize(c->stream));
  C3(cudaMemcpy(h, c->ke_out, sizeof h, cudaMemcpyDeviceToHost));
  if (ke) *ke = h[0];
  if (vol) *vol = h[1];
  return MST_OK;
}

mst_status mst_ctx3d_profile(mst_ctx3d* c, int on) {
  if (!c) return fail3(MST_EINVAL, "NULL context");
  drain3(c);
  c->profiling = on != 0;
  c->kname.clear();
  c->klaunch.clear();
  c->kms.clear();
  return MST_OK;
}

int mst_ctx3d_profile_count(mst_ctx3d* c) { return c ? (int)c->kname.size() : 0; }

mst_status mst_ctx3d_profile_get(mst_ctx3d* c, int i, char* name, size_t name_len, int* launches,
                                 double* total_ms) {
  if (!c || i < 0 || i >= (int)c->kname.size()) return fail3(MST_EINVAL, "bad kernel index");
  drain3(c);
  if (name && name_len) {
    std::strncpy(name, c->kname[i].c_str(), name_len - 1);
    name[name_len - 1] = 0;
  }
  if (launches) *launches = c->klaunch[i];
  if (total_ms) *total_ms = c->kms[i];
  return MST_OK;
}

}  // extern "C"
