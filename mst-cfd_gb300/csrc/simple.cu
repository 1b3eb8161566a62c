// Pressure-based SIMPLE solver of the reference (pSolver/SolverSIMPLE.cpp,
// the PSOLVER its CONST.h selects) on the GPU, bit-identical to the
// reference's arithmetic (compiled with --fmad=false).
//
// One time step = PSolver::solve (pSolver/PSolver.cpp:19-24) = SIMPLE_INTERVAL
// iterations of SolverSIMPLE::solve (:48-80):
//   face pass        updateFacePUVT (:82-193): central face (p,u,v,T) by zone
//   momentum         updateUStar / updateVStar (:247-439): one matrix, two
//                    right sides (the density reads p and T only, which the
//                    u solve does not change), Gauss-Seidel on both at once
//   face pass        again, with the new u and v
//   pressure         updatePUV2 (:712-838): p' system, Gauss-Seidel,
//                    p += SIMPLE_ALPHA_P p'
//   energy           updateT (:1315-1346), explicit
//   residual         max |new - old_n| / (old_n + EOR) (:62-71); after the
//                    last iteration also the Time loop's row (time/Time.cpp:66-72)
// updateGrad and updateFacePUVTRhieChow run in the reference too, but what
// they write is read nowhere on this path; they are not executed.
//
// Gauss-Seidel (lusolver/SparseSolverNUM.cpp:214-252): the reference walks
// its column lists in insertion order; row-wise, the same contributions
// reach each row in (column ascending, insertion) order.  Rows of one level
// of the forward sweep are independent.  The matrix structure is fixed by
// the mesh (insertion order: inner, then bond2, then bond1 cells, each
// cell's faces in order), so it is built once on the host together with the
// slot every cell-face coefficient is written to.
//
// GB300 mapping: the meshes this path runs on are small (thousands to tens
// of thousands of cells) and every SIMPLE iteration is a chain of ~100
// dependent phases (face passes, assembly, the Gauss-Seidel levels), so a
// whole time step is ONE persistent kernel on one thread-block cluster (up
// to 16 CTAs of 512 threads), the phases separated by the hardware cluster
// barrier instead of kernel launches.  Arrays written inside the kernel are
// read with ld.global.cg (L2), so no SM reads a stale L1 line.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "ctx.hpp"

namespace cg = cooperative_groups;

namespace {

constexpr int kThreads = 512;
constexpr int kLuInterval = 5;               // LU_INTERVAL (include/CONST.h:57)
constexpr double kCpCv = 1002.12 - 715.8;    // (CP - CV)
constexpr double kInvCp = 1 / 1002.12;       // 1 / CP
constexpr double kEor = 1e-10;               // EOR
constexpr int kPart = 8;                     // scratch doubles per CTA

// (p, u, v, T) of a cell or face, 32 bytes, read and written as two
// 16-byte halves
struct alignas(16) Puvt {
  double x, y, z, w;
};

struct SimpleDev {
  int nC, n_inner, nF;
  double dt, alpha_p;
  int wall_smooth;
  double inlet[4], p_out;
  // mesh, file order
  const int *c_ptr, *c_faces, *c_nb;
  const double2* c_dof;
  const double *c_eta, *c_vol;
  const double2* c_ctr;
  const unsigned char* c_cls;  // 0 inner, 1 bond2, 2 bond1
  const int2* f_cells;
  const int* f_type;
  const double* f_eta;
  const double2* f_dxy;        // wall faces: node1 - node0
  // systems: slot per cell-face (>= 0: L value index, <= -2: U value index
  // -(s+2), -1: not in the matrix)
  const int *m_slot, *p_slot;
  const int *ml_ptr, *ml_col, *mu_ptr, *mu_col, *m_lev_ptr, *m_lev_rows;
  const int *pl_ptr, *pl_col, *pu_ptr, *pu_col, *p_lev_ptr, *p_lev_rows;
  int n_m_levels, n_p_levels;
  double *ml_val, *mu_val, *pl_val, *pu_val;
  double *Dm, *Dp, *bu, *bv, *bp, *xu, *xv, *xp, *ru, *rv, *rp;
  double *wm, *wp;        // per solve: L value * (1 / D[column]) (forward sweep)
  double *Dim, *Dip;      // per solve: 1 / D
  Puvt *puvt, *oldn, *face;
  double* rho_f;          // [nF] density of the face values (face pass)
  double* rho_o;          // [nC] density of the old time level
  const double *cf_dist, *cf_dn;  // [tot] |x_c - x_nb| and |S| per cell-face
  double* part;           // [cluster CTAs][kPart]
  double* time_rows;      // [steps][4]
  double* inner_rows;     // [steps][n_inner][4]
  int* gs_iters;          // [steps][n_inner][3]
};

__device__ __forceinline__ Puvt mk(double x, double y, double z, double w) {
  Puvt v;
  v.x = x, v.y = y, v.z = z, v.w = w;
  return v;
}
__device__ __forceinline__ double ldc(const double* p) { return __ldcg(p); }
__device__ __forceinline__ Puvt ldc4(const Puvt* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldcg(q), b = __ldcg(q + 1);
  return mk(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void st4(Puvt* p, Puvt v) {
  double2* q = reinterpret_cast<double2*>(p);
  q[0] = make_double2(v.x, v.y);
  q[1] = make_double2(v.z, v.w);
}
__device__ __forceinline__ double comp(const Puvt& v, int k) {
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

// getPBasedRho (work/FUNCTION.cpp:25-27)
__device__ __forceinline__ double rho_pb(const Puvt& x) { return x.x / kCpCv / x.w; }

// running maximum that never takes a NaN (the reference's `if (r < q) r = q`)
__device__ __forceinline__ double dmax(double m, double q) { return (m < q) ? q : m; }

__device__ __forceinline__ void cluster_sync() { cg::this_cluster().sync(); }

// CTA maximum of K values into part[CTA rank in the cluster][0..K); callers
// cluster_sync()
// before reading the partials
template <int K>
__device__ void cta_max(double (&v)[K], double* part) {
  __shared__ double red[kThreads / 32][K];
  for (int k = 0; k < K; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] = dmax(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < K; ++k) red[threadIdx.x >> 5][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < K; ++k) {
      double m = red[0][k];
      for (int w = 1; w < kThreads / 32; ++w) m = dmax(m, red[w][k]);
      part[kPart * cg::this_cluster().block_rank() + k] = m;
    }
}
__device__ __forceinline__ double all_max(const double* part, int k) {
  double m = ldc(part + k);
  const int nb = (int)cg::this_cluster().num_blocks();
  for (int b = 1; b < nb; ++b) m = dmax(m, ldc(part + kPart * b + k));
  return m;
}

// ---- updateFacePUVT (:82-193) ------------------------------------------------
__device__ void face_pass(const SimpleDev& S, int gtid, int gstride) {
  for (int f = gtid; f < S.nF; f += gstride) {
    const int t = S.f_type[f];
    const int2 cc = S.f_cells[f];
    Puvt v;
    if (t == 2) {
      const Puvt a = ldc4(S.puvt + cc.x), b = ldc4(S.puvt + cc.y);
      const double e = S.f_eta[f];
      v = mk(a.x * e + (1 - e) * b.x, a.y * e + (1 - e) * b.y, a.z * e + (1 - e) * b.z,
             a.w * e + (1 - e) * b.w);
    } else if (t == 10) {
      v = mk(S.inlet[0], S.inlet[1], S.inlet[2], S.inlet[3]);
    } else if (t == 3) {
      const Puvt in = ldc4(S.puvt + cc.x);
      const double2 d = S.f_dxy[f];
      const double dX = d.x, dY = d.y;
      double o1 = 0, o2 = 0;
      if (S.wall_smooth) {
        o2 = (2 * dX * dY * in.y - (dX * dX - dY * dY) * in.z) / (dX * dX + dY * dY);
        o1 = (2 * dX * dY * in.z - (dY * dY - dX * dX) * in.y) / (dX * dX + dY * dY);
      }
      v = mk((in.x + in.x) / 2.0, (o1 + in.y) / 2.0, (o2 + in.z) / 2.0, (in.w + in.w) / 2.0);
    } else if (t == 5) {
      const Puvt in = ldc4(S.puvt + cc.x);
      v = mk(S.p_out, in.y, in.z, in.w);
    } else {
      v = ldc4(S.face + f);  // other zone types keep their values (the reference skips them)
    }
    if (t == 2 || t == 10 || t == 3 || t == 5) st4(S.face + f, v);
    // the density of the face value, formed once here for every reader
    S.rho_f[f] = rho_pb(v);
  }
}

__device__ __forceinline__ void put(double* lv, double* uv, int slot, double v) {
  if (slot >= 0) lv[slot] = v;
  else uv[-(slot + 2)] = v;
}

// ---- updateUStar / updateVStar (:247-439) ------------------------------------
__device__ void momentum(const SimpleDev& S, int gtid, int gstride) {
  for (int c = gtid; c < S.nC; c += gstride) {
    const int cls = S.c_cls[c];
    const double V = S.c_vol[c];
    const Puvt pc = ldc4(S.puvt + c), o = ldc4(S.oldn + c);
    double cofC = rho_pb(pc) * V / S.dt;
    const double ro = ldc(S.rho_o + c);
    const double rtu = (cls == 0) ? ro * o.y * V / S.dt : ro * V * o.y / S.dt;
    const double rtv = ro * V * o.z / S.dt;
    double rpu = 0, rpv = 0, rbu = 0, rbv = 0;
    for (int j = S.c_ptr[c]; j < S.c_ptr[c + 1]; ++j) {
      const int f = S.c_faces[j];
      const Puvt x = ldc4(S.face + f);
      const double2 d = S.c_dof[j];
      const double rf = ldc(S.rho_f + f);
      const int slot = S.m_slot[j];
      if (slot != -1) {
        const double e = S.c_eta[j];
        double t = (rf * x.y) * d.x;
        t += (rf * x.z) * d.y;
        cofC += t * e;
        put(S.ml_val, S.mu_val, slot, t * (1 - e));
      } else {
        const double su = -rf * x.y, sv = -rf * x.z;
        double tu = (su * x.y) * d.x;
        tu += (su * x.z) * d.y;
        double tv = (sv * x.y) * d.x;
        tv += (sv * x.z) * d.y;
        rbu += tu;
        rbv += tv;
      }
      rpu += -x.x * d.x;
      rpv += -x.x * d.y;
    }
    S.Dm[c] = cofC;
    S.bu[c] = (cls == 2) ? rpu + rtu + rbu : rpu + rtu;
    S.bv[c] = (cls == 2) ? rpv + rtv + rbv : rpv + rtv;
    S.xu[c] = pc.y;
    S.xv[c] = pc.z;
  }
}

// ---- updatePUV2 (:712-838) ---------------------------------------------------
__device__ void pressure(const SimpleDev& S, int gtid, int gstride) {
  for (int c = gtid; c < S.nC; c += gstride) {
    const int cls = S.c_cls[c];
    const double V = S.c_vol[c];
    const Puvt pc = ldc4(S.puvt + c), o = ldc4(S.oldn + c);
    const double Dc = ldc(S.Dm + c);
    double cofPC = V / S.dt / kCpCv / pc.w;
    double rhs = -V * (rho_pb(pc) - ldc(S.rho_o + c)) / S.dt;
    for (int j = S.c_ptr[c]; j < S.c_ptr[c + 1]; ++j) {
      const int f = S.c_faces[j];
      const Puvt x = ldc4(S.face + f);
      const double2 d = S.c_dof[j];
      const double rf = ldc(S.rho_f + f);
      const double dot = x.y * d.x + x.z * d.y;
      rhs += -rf * dot;
      const int slot = S.p_slot[j];
      if (slot == -1) continue;
      const double e = S.c_eta[j];
      const int F = S.c_nb[j];
      const double dist = S.cf_dist[j], dn = S.cf_dn[j];
      // the u and v diagonals are equal; both coefficients divide the
      // neighbour's volume by the u diagonal (:733-734)
      const double a = e * V / Dc + (1 - e) * S.c_vol[F] / ldc(S.Dm + F);
      const double cu = a / dist * d.x / dn;
      const double cv = a / dist * d.y / dn;
      cofPC += e * rf / pc.x * dot;
      double cofPF = (1 - e) * rf / pc.x * dot;
      cofPC += rf * (cu * d.x + cv * d.y);
      cofPF += -rf * (cu * d.x + cv * d.y);
      put(S.pl_val, S.pu_val, slot, cofPF);
    }
    // addD on a zero diagonal for inner and bond2 cells, setD for bond1
    S.Dp[c] = (cls == 2) ? cofPC : 0.0 + cofPC;
    S.bp[c] = rhs;
    S.xp[c] = 0.0;
  }
}

// ---- SparseSolverNUM::solveGS (lusolver/SparseSolverNUM.cpp:214-252) ---------
// A thread's first row of one sweep level: its first kPre lower entries
// (column, L / D[column]) and its own RHS
constexpr int kPre = 4;
template <int NS>
struct SweepRow {
  int row, k0, k1;
  int c[kPre];
  double w[kPre];
  double rr[NS];
};
template <int NS>
__device__ __forceinline__ void sweep_fetch(SweepRow<NS>& p, int l, const int* lev_ptr,
                                            const int* lev_rows, const int* l_ptr,
                                            const int* l_col, const double* w,
                                            double* const* r, const bool* done, int gtid) {
  const int i = lev_ptr[l] + gtid;
  p.row = (i < lev_ptr[l + 1]) ? lev_rows[i] : -1;
  if (p.row < 0) return;
  p.k0 = l_ptr[p.row];
  p.k1 = l_ptr[p.row + 1];
#pragma unroll
  for (int t = 0; t < kPre; ++t)
    if (p.k0 + t < p.k1) {
      p.c[t] = l_col[p.k0 + t];
      p.w[t] = ldc(w + p.k0 + t);
    }
  for (int s = 0; s < NS; ++s)
    if (!done[s]) p.rr[s] = ldc(r[s] + p.row);
}

// NS right-hand sides of one matrix; its[s] receives the iterations run.
template <int NS>
__device__ void gauss_seidel(const SimpleDev& S, const int* u_ptr, const int* u_col,
                             const double* u_val, const int* l_ptr, const int* l_col,
                             const double* l_val, const int* lev_ptr, const int* lev_rows,
                             int n_levels, const double* D, double* Di, double* w,
                             double* const* b, double* const* x,
                             double* const* r, int* its, int gtid, int gstride) {
  bool done[NS];
  for (int s = 0; s < NS; ++s) done[s] = false, its[s] = kLuInterval;
  // 1 / D and the forward sweep's L (1 / D[column]) once per solve: the
  // reference forms the same quotients and products in every iteration
  for (int row = gtid; row < S.nC; row += gstride) {
    Di[row] = 1. / ldc(D + row);
    for (int k = l_ptr[row]; k < l_ptr[row + 1]; ++k)
      w[k] = (ldc(l_val + k)) * (1. / ldc(D + l_col[k]));
  }
  cluster_sync();
  for (int it = 0; it < kLuInterval; ++it) {
    // RHS = RHSb - sum_U U X
    for (int row = gtid; row < S.nC; row += gstride)
      for (int s = 0; s < NS; ++s) {
        if (done[s]) continue;
        double acc = 0.;
        for (int k = u_ptr[row]; k < u_ptr[row + 1]; ++k) acc += ldc(u_val + k) * ldc(x[s] + u_col[k]);
        r[s][row] = ldc(b[s] + row) - acc;
      }
    cluster_sync();
    // forward sweep, level by level (level 0 rows have no lower entries).
    // A thread's first row of level l+1 (its entries' columns and weights,
    // and its own RHS, which only its level changes) is fetched while level
    // l runs; after the barrier only the RHS of earlier rows is loaded.
    SweepRow<NS> cur, nxt;
    if (n_levels > 1) sweep_fetch<NS>(cur, 1, lev_ptr, lev_rows, l_ptr, l_col, w, r, done, gtid);
    for (int l = 1; l < n_levels; ++l) {
      if (l + 1 < n_levels)
        sweep_fetch<NS>(nxt, l + 1, lev_ptr, lev_rows, l_ptr, l_col, w, r, done, gtid);
      if (cur.row >= 0)
        for (int s = 0; s < NS; ++s) {
          if (done[s]) continue;
          double acc = cur.rr[s];
#pragma unroll
          for (int t = 0; t < kPre; ++t)
            if (cur.k0 + t < cur.k1) acc -= cur.w[t] * ldc(r[s] + cur.c[t]);
          for (int k = cur.k0 + kPre; k < cur.k1; ++k) acc -= ldc(w + k) * ldc(r[s] + l_col[k]);
          r[s][cur.row] = acc;
        }
      for (int i = lev_ptr[l] + gtid + gstride; i < lev_ptr[l + 1]; i += gstride) {
        const int row = lev_rows[i];
        for (int s = 0; s < NS; ++s) {
          if (done[s]) continue;
          double acc = ldc(r[s] + row);
          for (int k = l_ptr[row]; k < l_ptr[row + 1]; ++k) acc -= ldc(w + k) * ldc(r[s] + l_col[k]);
          r[s][row] = acc;
        }
      }
      cluster_sync();
      cur = nxt;
    }
    // X = D^-1 RHS and the largest |X - X'| / X
    double m[NS];
    for (int s = 0; s < NS; ++s) m[s] = 0.;
    for (int row = gtid; row < S.nC; row += gstride)
      for (int s = 0; s < NS; ++s) {
        if (done[s]) continue;
        const double xn = ldc(Di + row) * ldc(r[s] + row);
        const double xo = ldc(x[s] + row);
        m[s] = dmax(m[s], fabs(xo - xn) / xo);
        x[s][row] = xn;
      }
    cta_max<NS>(m, S.part);
    cluster_sync();
    bool all = true;
    for (int s = 0; s < NS; ++s) {
      if (!done[s]) {
        const double res = all_max(S.part, s);
        if (res > 1e-10 * 1e-10 && res < 1e-7) done[s] = true, its[s] = it + 1;
      }
      all = all && done[s];
    }
    if (all) break;
  }
}

// p += alpha p', updateT (:1315-1346), the residual rows; on the last
// iteration of a step the old time level becomes the new state
__device__ void energy_and_residual(const SimpleDev& S, bool last, double (&res)[8], int gtid,
                                    int gstride) {
  for (int k = 0; k < 8; ++k) res[k] = 0.;
  for (int c = gtid; c < S.nC; c += gstride) {
    Puvt x = ldc4(S.puvt + c);
    const Puvt o = ldc4(S.oldn + c);
    x.x += S.alpha_p * ldc(S.xp + c);
    double rhs = 0;
    for (int j = S.c_ptr[c]; j < S.c_ptr[c + 1]; ++j) {
      const int f = S.c_faces[j];
      const Puvt s4 = ldc4(S.face + f);
      const double2 d = S.c_dof[j];
      rhs += -ldc(S.rho_f + f) * s4.w * (d.x * s4.y + d.y * s4.z);
      rhs += kInvCp * s4.x * (d.x + d.y);
    }
    x.w = (rhs / S.c_vol[c] * S.dt + kInvCp * (x.x - o.x) + ldc(S.rho_o + c) * o.w) / rho_pb(x);
    st4(S.puvt + c, x);
    for (int k = 0; k < 4; ++k) {
      const double dn = fabs(comp(x, k) - comp(o, k));
      res[k] = dmax(res[k], dn / (comp(o, k) + kEor));
      if (last) res[4 + k] = dmax(res[4 + k], dn / comp(o, k));
    }
    if (last) {
      st4(S.oldn + c, x);
      S.rho_o[c] = rho_pb(x);
    }
  }
}

// nsteps time steps of one case on one thread-block cluster
__device__ void simple_steps(const SimpleDev& S, int nsteps) {
  const int gtid = (int)cg::this_cluster().block_rank() * blockDim.x + threadIdx.x;
  const int gstride = (int)cg::this_cluster().num_blocks() * blockDim.x;
  const bool writer = (gtid == 0);
  for (int step = 0; step < nsteps; ++step) {
    for (int it = 0; it < S.n_inner; ++it) {
      const bool last = (it == S.n_inner - 1);
      int its[3];
      face_pass(S, gtid, gstride);
      cluster_sync();
      momentum(S, gtid, gstride);
      cluster_sync();
      {
        double* const b[2] = {S.bu, S.bv};
        double* const x[2] = {S.xu, S.xv};
        double* const r[2] = {S.ru, S.rv};
        gauss_seidel<2>(S, S.mu_ptr, S.mu_col, S.mu_val, S.ml_ptr, S.ml_col, S.ml_val,
                        S.m_lev_ptr, S.m_lev_rows, S.n_m_levels, S.Dm, S.Dim, S.wm, b, x, r, its, gtid,
                        gstride);
      }
      for (int c = gtid; c < S.nC; c += gstride) {
        Puvt v = ldc4(S.puvt + c);
        v.y = ldc(S.xu + c);
        v.z = ldc(S.xv + c);
        st4(S.puvt + c, v);
      }
      cluster_sync();
      face_pass(S, gtid, gstride);
      cluster_sync();
      pressure(S, gtid, gstride);
      cluster_sync();
      {
        double* const b[1] = {S.bp};
        double* const x[1] = {S.xp};
        double* const r[1] = {S.rp};
        gauss_seidel<1>(S, S.pu_ptr, S.pu_col, S.pu_val, S.pl_ptr, S.pl_col, S.pl_val,
                        S.p_lev_ptr, S.p_lev_rows, S.n_p_levels, S.Dp, S.Dip, S.wp, b, x, r, its + 2, gtid,
                        gstride);
      }
      double res[8];
      energy_and_residual(S, last, res, gtid, gstride);
      cta_max<8>(res, S.part);
      cluster_sync();
      if (writer) {
        const size_t row = (size_t)step * S.n_inner + it;
        for (int k = 0; k < 4; ++k) S.inner_rows[4 * row + k] = all_max(S.part, k);
        for (int k = 0; k < 3; ++k) S.gs_iters[3 * row + k] = its[k];
        if (last)
          for (int k = 0; k < 4; ++k) S.time_rows[4 * (size_t)step + k] = all_max(S.part, 4 + k);
      }
      // the partials are rewritten only after the next face pass's barrier
    }
  }
}

__global__ void __launch_bounds__(kThreads, 1) k_simple_steps(SimpleDev S, int nsteps) {
  simple_steps(S, nsteps);
}

// Independent cases, one cluster each (cluster c runs devs[c]); clusters
// never wait on one another.
__global__ void __launch_bounds__(kThreads, 1) k_simple_steps_batch(const SimpleDev* devs,
                                                                     int nsteps) {
  __shared__ SimpleDev S;
  const int c = blockIdx.x / (int)cg::this_cluster().num_blocks();
  if (threadIdx.x == 0) S = devs[c];
  __syncthreads();
  simple_steps(S, nsteps);
}

// ---- host-side structure -------------------------------------------------------
struct Sys {
  std::vector<int> l_ptr, l_col, u_ptr, u_col, lev_ptr, lev_rows, slot;
  int n_levels = 0;
};

// in(c, j): whether cell-face j of cell c enters the matrix
template <class In>
bool build_sys(const mst::HostMesh& h, const std::vector<unsigned char>& cls, In in, Sys* s) {
  const int nC = h.n_cells, tot = (int)h.cell_faces.size();
  s->slot.assign(tot, -1);
  std::vector<std::vector<std::pair<int, int>>> lrow(nC), urow(nC);  // (col, cell-face)
  for (int c = 0; c < nC; ++c)
    for (int j = h.cell_ptr[c]; j < h.cell_ptr[c + 1]; ++j) {
      if (!in(c, j, cls[c])) continue;
      const int nb = h.cell_nb[j];
      if (nb == c || nb < 0 || nb >= nC) return false;
      (nb < c ? lrow : urow)[c].push_back({nb, j});
    }
  auto pack = [&](std::vector<std::vector<std::pair<int, int>>>& rows, std::vector<int>* ptr,
                  std::vector<int>* col, bool lower) {
    ptr->assign(nC + 1, 0);
    col->clear();
    for (int c = 0; c < nC; ++c) {
      auto& v = rows[c];
      std::stable_sort(v.begin(), v.end(),
                       [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
                         return a.first < b.first;
                       });
      for (auto& e : v) {
        const int pos = (int)col->size();
        s->slot[e.second] = lower ? pos : -(pos + 2);
        col->push_back(e.first);
      }
      (*ptr)[c + 1] = (int)col->size();
    }
  };
  pack(lrow, &s->l_ptr, &s->l_col, true);
  pack(urow, &s->u_ptr, &s->u_col, false);
  std::vector<int> lev(nC, 0);
  int maxl = 0;
  for (int r = 0; r < nC; ++r) {
    int l = 0;
    for (int k = s->l_ptr[r]; k < s->l_ptr[r + 1]; ++k) l = std::max(l, lev[s->l_col[k]] + 1);
    lev[r] = l;
    maxl = std::max(maxl, l);
  }
  s->n_levels = maxl + 1;
  s->lev_ptr.assign(maxl + 2, 0);
  for (int r = 0; r < nC; ++r) s->lev_ptr[lev[r] + 1]++;
  for (int l = 0; l <= maxl; ++l) s->lev_ptr[l + 1] += s->lev_ptr[l];
  s->lev_rows.assign(nC, 0);
  std::vector<int> fill(s->lev_ptr.begin(), s->lev_ptr.end() - 1);
  for (int r = 0; r < nC; ++r) s->lev_rows[fill[lev[r]]++] = r;
  return true;
}

mst_status sfail(mst_status s, const std::string& m) { return mst_internal_fail(s, m); }

#define S_CU(call)                                                                  \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return sfail(MST_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// getP / getT (work/FUNCTION.cpp:7-14)
double q_p(const double* q) {
  return (q[3] - 0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0]) * (1.4 - 1);
}
double q_t(const double* q) {
  return (q[3] - 0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0]) / q[0] / 715.8;
}

}  // namespace

struct mst_simple {
  int nC = 0, nF = 0, cluster = 1;
  mst_simple_params prm{};
  cudaStream_t stream = nullptr;
  SimpleDev dv{};
  std::vector<void*> allocs;
  int rows_cap = 0;
  double *time_rows = nullptr, *inner_rows = nullptr;
  int* gs_iters = nullptr;
  int last_steps = 0;
  int m_levels = 0, p_levels = 0;
  std::vector<double> rho_host;
  int last_batch_cluster = 0;
};

namespace {

template <class T>
cudaError_t sup(mst_simple* s, T** dst, const std::vector<T>& v, size_t n = 0) {
  const size_t cnt = std::max<size_t>(std::max(v.size(), n), 1);
  cudaError_t e = cudaMalloc((void**)dst, cnt * sizeof(T));
  if (e != cudaSuccess) return e;
  s->allocs.push_back(*dst);
  if (!v.empty()) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  else e = cudaMemset(*dst, 0, cnt * sizeof(T));
  return e;
}

mst_status ensure_rows(mst_simple* s, int nsteps) {
  if (nsteps <= s->rows_cap) return MST_OK;
  for (void* p : {(void*)s->time_rows, (void*)s->inner_rows, (void*)s->gs_iters}) {
    if (!p) continue;
    cudaFree(p);
    s->allocs.erase(std::remove(s->allocs.begin(), s->allocs.end(), p), s->allocs.end());
  }
  const int cap = std::max(nsteps, 16);
  const size_t ni = (size_t)cap * s->prm.n_inner;
  S_CU(cudaMalloc((void**)&s->time_rows, (size_t)cap * 4 * sizeof(double)));
  s->allocs.push_back(s->time_rows);
  S_CU(cudaMalloc((void**)&s->inner_rows, ni * 4 * sizeof(double)));
  s->allocs.push_back(s->inner_rows);
  S_CU(cudaMalloc((void**)&s->gs_iters, ni * 3 * sizeof(int)));
  s->allocs.push_back(s->gs_iters);
  s->rows_cap = cap;
  s->dv.time_rows = s->time_rows;
  s->dv.inner_rows = s->inner_rows;
  s->dv.gs_iters = s->gs_iters;
  return MST_OK;
}

// largest cluster (16, 8, 4, 2, 1 CTAs) the device can place
int pick_cluster(int want) {
  cudaFuncSetAttribute(k_simple_steps, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  for (int nb : {16, 8, 4, 2, 1}) {
    if (want > 0 && nb > want) continue;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    cfg.gridDim = dim3(nb);
    cfg.blockDim = dim3(kThreads);
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = nb;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_simple_steps, &cfg) == cudaSuccess && n > 0)
      return nb;
    cudaGetLastError();
  }
  return 0;
}

}  // namespace

extern "C" {

mst_status mst_simple_default_params(mst_simple_params* p) {
  if (!p) return sfail(MST_EINVAL, "NULL params");
  std::memset(p, 0, sizeof *p);
  // the reference's initial state (CONST.h:70-83): rho = 1, u = v = 0,
  // E = rho (T CV + 0.5 |u|^2), T = 1/286.32
  const double T = 1 / 286.32;
  const double q[4] = {1, 1.0 * 0, 1.0 * 0, 1 * (T * 715.8 + 0.5 * (0 * 0 + 0 * 0))};
  p->dt = 1. / 4e+3;  // 1 / STEP_TIME
  p->alpha_p = 0.3;   // SIMPLE_ALPHA_P
  p->n_inner = 5;     // SIMPLE_INTERVAL
  p->wall_smooth = 1; // FLAG_WALLSMOOTH
  p->inlet[0] = q_p(q);
  p->inlet[1] = 0;
  p->inlet[2] = 0;
  p->inlet[3] = T;
  p->p_out = q_p(q);
  p->cluster = 0;
  return MST_OK;
}

mst_status mst_q_to_puvt(int n, const double* q, double* puvt) {
  if (n < 0 || (n > 0 && (!q || !puvt))) return sfail(MST_EINVAL, "bad arguments");
  for (int i = 0; i < n; ++i) {
    const double* a = q + 4 * (size_t)i;
    double* o = puvt + 4 * (size_t)i;
    o[0] = q_p(a);
    o[1] = a[1] / a[0];
    o[2] = a[2] / a[0];
    o[3] = q_t(a);
  }
  return MST_OK;
}

mst_status mst_simple_create(const mst_mesh* mesh, const mst_simple_params* prm,
                             mst_simple** out) {
  if (!mesh || !out) return sfail(MST_EINVAL, "NULL argument");
  *out = nullptr;
  mst_simple_params p;
  if (prm) p = *prm;
  else mst_simple_default_params(&p);
  if (p.n_inner < 1 || p.cluster < 0 || p.cluster > 16)
    return sfail(MST_EINVAL, "n_inner must be >= 1 and cluster in 0..16");
  const mst::HostMesh& h = mesh->host;
  if (!h.c1_shift.empty())
    return sfail(MST_EUNSUPPORTED, "periodic meshes are not part of the SIMPLE path");
  const int nC = h.n_cells, nF = h.n_faces;
  if (nC <= 0) return sfail(MST_EMESH, "empty mesh");
  std::vector<unsigned char> cls(nC, 0);
  for (int c : h.bond2) cls[c] = 1;
  for (int c : h.bond1) cls[c] = 2;
  Sys ms, ps;
  const bool ok_m = build_sys(
      h, cls,
      [&](int, int j, int k) { return k != 2 || h.cell_faces[j] < h.n_int_faces; }, &ms);
  const bool ok_p = build_sys(
      h, cls, [&](int, int j, int k) { return k != 2 || h.face_type[h.cell_faces[j]] == 2; },
      &ps);
  if (!ok_m || !ok_p) return sfail(MST_EMESH, "a matrix face joins a cell to itself");
  for (int f = 0; f < nF; ++f)
    if (h.face_type[f] == 2 && h.face_cells[2 * f + 1] < 0)
      return sfail(MST_EMESH, "interior face without a second cell");

  auto s = new (std::nothrow) mst_simple;
  if (!s) return sfail(MST_ENOMEM, "host allocation failed");
  s->nC = nC;
  s->nF = nF;
  s->prm = p;
  s->cluster = pick_cluster(p.cluster);
  if (s->cluster == 0) {
    delete s;
    return sfail(MST_ECUDA, "no thread-block cluster of the SIMPLE kernel fits this device");
  }
  s->m_levels = ms.n_levels;
  s->p_levels = ps.n_levels;

  std::vector<double2> dof(h.cell_dof.size() / 2), ctr(nC), dxy(nF);
  for (size_t j = 0; j < dof.size(); ++j) dof[j] = make_double2(h.cell_dof[2 * j], h.cell_dof[2 * j + 1]);
  for (int c = 0; c < nC; ++c) ctr[c] = make_double2(h.cell_ctr[2 * c], h.cell_ctr[2 * c + 1]);
  std::vector<int2> fcells(nF);
  for (int f = 0; f < nF; ++f) {
    fcells[f] = make_int2(h.face_cells[2 * f], h.face_cells[2 * f + 1]);
    const int n0 = h.face_nodes[2 * f], n1 = h.face_nodes[2 * f + 1];
    dxy[f] = make_double2(h.node_xy[2 * n1] - h.node_xy[2 * n0],
                          h.node_xy[2 * n1 + 1] - h.node_xy[2 * n0 + 1]);
  }
  // |x_c - x_nb| and |S| per cell-face, as the pressure coefficients form them
  // (SolverSIMPLE.cpp:733-734: Eigen norm = sqrt(x0*x0 + x1*x1))
  const int tot = (int)h.cell_faces.size();
  std::vector<double> cdist(tot, 0.0), cdn(tot, 0.0);
  for (int c = 0; c < nC; ++c)
    for (int j = h.cell_ptr[c]; j < h.cell_ptr[c + 1]; ++j) {
      const int F = h.cell_nb[j];
      const double rx = h.cell_ctr[2 * c] - h.cell_ctr[2 * F];
      const double ry = h.cell_ctr[2 * c + 1] - h.cell_ctr[2 * F + 1];
      double sq = rx * rx;
      sq += ry * ry;
      cdist[j] = std::sqrt(sq);
      const double dx = h.cell_dof[2 * j], dy = h.cell_dof[2 * j + 1];
      double sd = dx * dx;
      sd += dy * dy;
      cdn[j] = std::sqrt(sd);
    }
  SimpleDev& d = s->dv;
  d.nC = nC;
  d.nF = nF;
  d.n_inner = p.n_inner;
  d.dt = p.dt;
  d.alpha_p = p.alpha_p;
  d.wall_smooth = p.wall_smooth;
  for (int k = 0; k < 4; ++k) d.inlet[k] = p.inlet[k];
  d.p_out = p.p_out;
  d.n_m_levels = ms.n_levels;
  d.n_p_levels = ps.n_levels;
  const std::vector<double> none;
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  auto upi = [&](const int** dst, const std::vector<int>& v) {
    int* p_ = nullptr;
    if (e == cudaSuccess) e = sup(s, &p_, v);
    *dst = p_;
  };
  upi(&d.c_ptr, h.cell_ptr);
  upi(&d.c_faces, h.cell_faces);
  upi(&d.c_nb, h.cell_nb);
  upi(&d.f_type, h.face_type);
  upi(&d.m_slot, ms.slot);
  upi(&d.p_slot, ps.slot);
  upi(&d.ml_ptr, ms.l_ptr);
  upi(&d.ml_col, ms.l_col);
  upi(&d.mu_ptr, ms.u_ptr);
  upi(&d.mu_col, ms.u_col);
  upi(&d.m_lev_ptr, ms.lev_ptr);
  upi(&d.m_lev_rows, ms.lev_rows);
  upi(&d.pl_ptr, ps.l_ptr);
  upi(&d.pl_col, ps.l_col);
  upi(&d.pu_ptr, ps.u_ptr);
  upi(&d.pu_col, ps.u_col);
  upi(&d.p_lev_ptr, ps.lev_ptr);
  upi(&d.p_lev_rows, ps.lev_rows);
  {
    double2 *a = nullptr, *b = nullptr, *c2 = nullptr;
    double *eta = nullptr, *vol = nullptr, *feta = nullptr;
    unsigned char* cl = nullptr;
    int2* fc = nullptr;
    if (e == cudaSuccess) e = sup(s, &a, dof);
    if (e == cudaSuccess) e = sup(s, &b, ctr);
    if (e == cudaSuccess) e = sup(s, &c2, dxy);
    if (e == cudaSuccess) e = sup(s, &eta, h.cell_eta0c);
    if (e == cudaSuccess) e = sup(s, &vol, h.cell_vol);
    if (e == cudaSuccess) e = sup(s, &feta, h.face_eta0);
    if (e == cudaSuccess) e = sup(s, &cl, cls);
    if (e == cudaSuccess) e = sup(s, &fc, fcells);
    d.c_dof = a, d.c_ctr = b, d.f_dxy = c2, d.c_eta = eta, d.c_vol = vol, d.f_eta = feta;
    d.c_cls = cl, d.f_cells = fc;
  }
  for (double** v : {&d.ml_val, &d.mu_val, &d.pl_val, &d.pu_val, &d.wm, &d.wp}) {
    size_t n = (v == &d.ml_val || v == &d.wm) ? ms.l_col.size()
             : (v == &d.mu_val) ? ms.u_col.size()
             : (v == &d.pl_val || v == &d.wp) ? ps.l_col.size() : ps.u_col.size();
    if (e == cudaSuccess) e = sup(s, v, none, n);
  }
  for (double** v : {&d.Dm, &d.Dp, &d.bu, &d.bv, &d.bp, &d.xu, &d.xv, &d.xp, &d.ru, &d.rv,
                     &d.rp, &d.Dim, &d.Dip, &d.rho_o})
    if (e == cudaSuccess) e = sup(s, v, none, (size_t)nC);
  if (e == cudaSuccess) e = sup(s, &d.rho_f, none, (size_t)nF);
  {
    double *dd = nullptr, *dn = nullptr;
    if (e == cudaSuccess) e = sup(s, &dd, cdist);
    if (e == cudaSuccess) e = sup(s, &dn, cdn);
    d.cf_dist = dd, d.cf_dn = dn;
  }
  {
    double *pv = nullptr, *od = nullptr, *fcv = nullptr;
    if (e == cudaSuccess) e = sup(s, &pv, none, (size_t)nC * 4);
    if (e == cudaSuccess) e = sup(s, &od, none, (size_t)nC * 4);
    if (e == cudaSuccess) e = sup(s, &fcv, none, (size_t)nF * 4);
    d.puvt = reinterpret_cast<Puvt*>(pv);
    d.oldn = reinterpret_cast<Puvt*>(od);
    d.face = reinterpret_cast<Puvt*>(fcv);
  }
  if (e == cudaSuccess) e = sup(s, &d.part, none, (size_t)16 * kPart);
  if (e != cudaSuccess) {
    mst_simple_destroy(s);
    return sfail(MST_ECUDA, std::string("mst_simple_create: ") + cudaGetErrorString(e));
  }
  if (mst_status st = ensure_rows(s, 16)) {
    mst_simple_destroy(s);
    return st;
  }
  *out = s;
  return MST_OK;
}

mst_status mst_simple_set_state(mst_simple* s, const double* cell_puvt, const double* face_puvt) {
  if (!s || !cell_puvt) return sfail(MST_EINVAL, "NULL argument");
  const size_t cb = (size_t)s->nC * 4 * sizeof(double);
  S_CU(cudaMemcpyAsync(s->dv.puvt, cell_puvt, cb, cudaMemcpyHostToDevice, s->stream));
  S_CU(cudaMemcpyAsync(s->dv.oldn, cell_puvt, cb, cudaMemcpyHostToDevice, s->stream));
  // density of the old time level: the quotient getPBasedRho forms
  s->rho_host.resize(s->nC);
  for (int c = 0; c < s->nC; ++c)
    s->rho_host[c] = cell_puvt[4 * c] / (1002.12 - 715.8) / cell_puvt[4 * c + 3];
  S_CU(cudaMemcpyAsync(s->dv.rho_o, s->rho_host.data(), (size_t)s->nC * sizeof(double),
                       cudaMemcpyHostToDevice, s->stream));
  if (face_puvt)
    S_CU(cudaMemcpyAsync(s->dv.face, face_puvt, (size_t)s->nF * 4 * sizeof(double),
                         cudaMemcpyHostToDevice, s->stream));
  S_CU(cudaStreamSynchronize(s->stream));
  return MST_OK;
}

mst_status mst_simple_get_state(mst_simple* s, double* cell_puvt, double* face_puvt) {
  if (!s) return sfail(MST_EINVAL, "NULL argument");
  if (cell_puvt)
    S_CU(cudaMemcpyAsync(cell_puvt, s->dv.puvt, (size_t)s->nC * 4 * sizeof(double),
                         cudaMemcpyDeviceToHost, s->stream));
  if (face_puvt)
    S_CU(cudaMemcpyAsync(face_puvt, s->dv.face, (size_t)s->nF * 4 * sizeof(double),
                         cudaMemcpyDeviceToHost, s->stream));
  S_CU(cudaStreamSynchronize(s->stream));
  return MST_OK;
}

mst_status mst_simple_step(mst_simple* s, int nsteps, double* time_rows) {
  if (!s || nsteps < 0) return sfail(MST_EINVAL, "bad arguments");
  if (nsteps == 0) return MST_OK;
  if (mst_status st = ensure_rows(s, nsteps)) return st;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  cfg.gridDim = dim3(s->cluster);
  cfg.blockDim = dim3(kThreads);
  cfg.stream = s->stream;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = s->cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  S_CU(cudaLaunchKernelEx(&cfg, k_simple_steps, s->dv, nsteps));
  s->last_steps = nsteps;
  if (time_rows)
    S_CU(cudaMemcpyAsync(time_rows, s->time_rows, (size_t)nsteps * 4 * sizeof(double),
                         cudaMemcpyDeviceToHost, s->stream));
  S_CU(cudaStreamSynchronize(s->stream));
  return MST_OK;
}

mst_status mst_simple_step_batch(mst_simple* const* cases, int n, int nsteps,
                                 double* time_rows) {
  if (!cases || n < 1 || nsteps < 0) return sfail(MST_EINVAL, "bad arguments");
  for (int i = 0; i < n; ++i)
    if (!cases[i]) return sfail(MST_EINVAL, "NULL case");
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (cases[i] == cases[j]) return sfail(MST_EINVAL, "a case is listed twice");
  if (nsteps == 0) return MST_OK;
  std::vector<SimpleDev> devs(n);
  for (int i = 0; i < n; ++i) {
    if (mst_status st = ensure_rows(cases[i], nsteps)) return st;
    S_CU(cudaStreamSynchronize(cases[i]->stream));
    devs[i] = cases[i]->dv;
  }
  mst_simple* s0 = cases[0];
  SimpleDev* d_devs = nullptr;
  S_CU(cudaMalloc((void**)&d_devs, sizeof(SimpleDev) * n));
  cudaError_t e = cudaMemcpyAsync(d_devs, devs.data(), sizeof(SimpleDev) * n,
                                  cudaMemcpyHostToDevice, s0->stream);
  // Cluster size for the batch (results do not depend on it): the one that
  // minimises waves x per-case time, the per-case time taken to fall as
  // 1/sqrt(CTAs) (measured: 16, 8, 4 CTAs -> 6.5, 8.1, 11.5 ms on 18k cells)
  int nb_best = s0->cluster;
  if (e == cudaSuccess) {
    cudaFuncSetAttribute(k_simple_steps_batch, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    double best = 1e300;
    for (int nb : {16, 8, 4, 2, 1}) {
      cudaLaunchConfig_t q = {};
      cudaLaunchAttribute qa[1];
      q.gridDim = dim3(nb * n);
      q.blockDim = dim3(kThreads);
      qa[0].id = cudaLaunchAttributeClusterDimension;
      qa[0].val.clusterDim.x = nb;
      qa[0].val.clusterDim.y = 1;
      qa[0].val.clusterDim.z = 1;
      q.attrs = qa;
      q.numAttrs = 1;
      int active = 0;
      if (cudaOccupancyMaxActiveClusters(&active, k_simple_steps_batch, &q) != cudaSuccess ||
          active < 1) {
        cudaGetLastError();
        continue;
      }
      const double cost = (double)((n + active - 1) / active) / std::sqrt((double)nb);
      if (cost < best * (1 - 1e-9)) best = cost, nb_best = nb;
    }
  }
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    cfg.gridDim = dim3(nb_best * n);
    cfg.blockDim = dim3(kThreads);
    cfg.stream = s0->stream;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = nb_best;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_simple_steps_batch, (const SimpleDev*)d_devs, nsteps);
    s0->last_batch_cluster = nb_best;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s0->stream);
  cudaFree(d_devs);
  if (e != cudaSuccess)
    return sfail(MST_ECUDA, std::string("mst_simple_step_batch: ") + cudaGetErrorString(e));
  for (int i = 0; i < n; ++i) {
    cases[i]->last_steps = nsteps;
    if (time_rows)
      S_CU(cudaMemcpy(time_rows + (size_t)4 * nsteps * i, cases[i]->time_rows,
                      (size_t)nsteps * 4 * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return MST_OK;
}

mst_status mst_simple_rows(mst_simple* s, double* inner_rows, int* gs_iters) {
  if (!s) return sfail(MST_EINVAL, "NULL argument");
  const size_t ni = (size_t)s->last_steps * s->prm.n_inner;
  if (inner_rows && ni)
    S_CU(cudaMemcpyAsync(inner_rows, s->inner_rows, ni * 4 * sizeof(double),
                         cudaMemcpyDeviceToHost, s->stream));
  if (gs_iters && ni)
    S_CU(cudaMemcpyAsync(gs_iters, s->gs_iters, ni * 3 * sizeof(int), cudaMemcpyDeviceToHost,
                         s->stream));
  S_CU(cudaStreamSynchronize(s->stream));
  return MST_OK;
}

mst_status mst_simple_get_info(const mst_simple* s, mst_simple_info* info) {
  if (!s || !info) return sfail(MST_EINVAL, "NULL argument");
  std::memset(info, 0, sizeof *info);
  info->n_cells = s->nC;
  info->n_faces = s->nF;
  info->cluster = s->cluster;
  info->threads = kThreads;
  info->momentum_levels = s->m_levels;
  info->pressure_levels = s->p_levels;
  info->last_steps = s->last_steps;
  info->batch_cluster = s->last_batch_cluster;
  return MST_OK;
}

mst_status mst_simple_destroy(mst_simple* s) {
  if (!s) return MST_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (void* p : s->allocs) cudaFree(p);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return MST_OK;
}

}  // extern "C"
