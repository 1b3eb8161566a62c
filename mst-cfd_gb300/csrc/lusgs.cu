// Level-scheduled sparse sweeps of the reference's lusolver on the GPU.
//
//   scalar  SparseSolverNUM (lusolver/SparseSolverNUM.cpp): setELE/addELE
//           :115-140, solveILUSGS :144-212, solveGS :214-252
//   block   SparseSolver<Matrix4d, Vector4d> (lusolver/SparseSolver.cpp):
//           setD/setL/setU :35-48, solveILU :53-104
//
// The reference walks column lists (insertion order, duplicates kept):
// columns ascending for the products and the forward sweep, descending for
// the backward sweep.  Row-oriented, the same contributions reach each row
// in the same order when a row's entries are sorted by (column ascending,
// insertion order) -- or (column descending, insertion order) for the
// backward sweep.  Rows whose dependencies are all in earlier levels are
// independent, so each level is one parallel launch and every row adds its
// terms sequentially in that order: the results are bit-identical to the
// reference's (compiled with --fmad=false; 4x4 blocks use the adjugate
// inverse and left-to-right products of the oracle's Eigen shim).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "ctx.hpp"

namespace {

constexpr int kLuInterval = 5;  // LU_INTERVAL (include/CONST.h:57)

// ---- 4x4 block arithmetic, row-major, the shim's order ------------------
__device__ __forceinline__ double det3(double a, double b, double c, double d, double e,
                                       double f, double g, double h, double i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}
__device__ void inv4(const double* m, double* inv) {
  double cof[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const int r0 = (i == 0) ? 1 : 0, r1 = (i <= 1) ? 2 : 1, r2 = (i <= 2) ? 3 : 2;
      const int c0 = (j == 0) ? 1 : 0, c1 = (j <= 1) ? 2 : 1, c2 = (j <= 2) ? 3 : 2;
      const double v = det3(m[4 * r0 + c0], m[4 * r0 + c1], m[4 * r0 + c2], m[4 * r1 + c0],
                            m[4 * r1 + c1], m[4 * r1 + c2], m[4 * r2 + c0], m[4 * r2 + c1],
                            m[4 * r2 + c2]);
      cof[4 * i + j] = ((i + j) & 1) ? -v : v;
    }
  double det = m[0] * cof[0];
  det += m[1] * cof[1];
  det += m[2] * cof[2];
  det += m[3] * cof[3];
  const double id = 1.0 / det;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) inv[4 * i + j] = cof[4 * j + i] * id;
}
__device__ __forceinline__ void mv4(const double* a, const double* x, double* y) {
  for (int i = 0; i < 4; ++i) {
    double s = a[4 * i] * x[0];
    s += a[4 * i + 1] * x[1];
    s += a[4 * i + 2] * x[2];
    s += a[4 * i + 3] * x[3];
    y[i] = s;
  }
}
__device__ __forceinline__ void mm4(const double* a, const double* b, double* c) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = a[4 * i] * b[j];
      s += a[4 * i + 1] * b[4 + j];
      s += a[4 * i + 2] * b[8 + j];
      s += a[4 * i + 3] * b[12 + j];
      c[4 * i + j] = s;
    }
}

// ---- kernels: B = 1 (scalar) or 4 (blocks) ---------------------------------
// Phase A: RHSUx[r] = sum_U U * X (then D^-1) ; GS: RHS = b - sum_U U * X
template <int B>
__global__ void k_upper_product(int dim, const int* __restrict__ ptr, const int* __restrict__ col,
                                const double* __restrict__ val, const double* __restrict__ x,
                                const double* __restrict__ D, const double* __restrict__ Di,
                                const double* __restrict__ b, double* __restrict__ out, int gs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= dim) return;
  if (B == 1) {
    double s = 0.;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) s += val[k] * x[col[k]];
    out[r] = gs ? b[r] - s : s / D[r];
  } else {
    double s[4] = {0., 0., 0., 0.}, t[4];
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
      mv4(val + 16 * (size_t)k, x + 4 * (size_t)col[k], t);
      for (int j = 0; j < 4; ++j) s[j] += t[j];
    }
    mv4(Di + 16 * (size_t)r, s, t);
    for (int j = 0; j < 4; ++j) out[4 * (size_t)r + j] = t[j];
  }
}

// Phase B: RHS[r] = b[r] + sum_L L * RHSUx
template <int B>
__global__ void k_lower_product(int dim, const int* __restrict__ ptr, const int* __restrict__ col,
                                const double* __restrict__ val, const double* __restrict__ y,
                                const double* __restrict__ b, double* __restrict__ rhs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= dim) return;
  double s[B], t[4];
  for (int j = 0; j < B; ++j) s[j] = 0.;
  for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
    if (B == 1) {
      s[0] += val[k] * y[col[k]];
    } else {
      mv4(val + 16 * (size_t)k, y + 4 * (size_t)col[k], t);
      for (int j = 0; j < B; ++j) s[j] += t[j];
    }
  }
  for (int j = 0; j < B; ++j) rhs[B * (size_t)r + j] = b[B * (size_t)r + j] + s[j];
}

// One level of a sweep: v[r] -= (M * D^-1[k]) * v[k] over the row's entries
// in order (forward: L, columns ascending; backward: U, columns descending)
template <int B>
__global__ void k_sweep_level(int n, const int* __restrict__ rows, const int* __restrict__ ptr,
                              const int* __restrict__ col, const double* __restrict__ val,
                              const double* __restrict__ D, const double* __restrict__ Di,
                              double* __restrict__ v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = rows[i];
  if (B == 1) {
    double acc = v[r];
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
      const int c = col[k];
      acc -= (val[k]) * (1. / D[c]) * v[c];
    }
    v[r] = acc;
  } else {
    double acc[4], M[16], t[4];
    for (int j = 0; j < 4; ++j) acc[j] = v[4 * (size_t)r + j];
    for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
      const int c = col[k];
      mm4(val + 16 * (size_t)k, Di + 16 * (size_t)c, M);
      mv4(M, v + 4 * (size_t)c, t);
      for (int j = 0; j < 4; ++j) acc[j] -= t[j];
    }
    for (int j = 0; j < 4; ++j) v[4 * (size_t)r + j] = acc[j];
  }
}

// X1 = D^-1 RHS ; RHS1 = D X1
template <int B>
__global__ void k_middle(int dim, const double* __restrict__ D, const double* __restrict__ Di,
                         const double* __restrict__ rhs, double* __restrict__ rhs1) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= dim) return;
  if (B == 1) {
    const double x1 = (1. / D[r]) * rhs[r];
    rhs1[r] = D[r] * x1;
  } else {
    double x1[4], t[4];
    mv4(Di + 16 * (size_t)r, rhs + 4 * (size_t)r, x1);
    mv4(D + 16 * (size_t)r, x1, t);
    for (int j = 0; j < 4; ++j) rhs1[4 * (size_t)r + j] = t[j];
  }
}

// X = D^-1 v and, for the scalar solver, the largest |X - X'| / X (signed
// division and NaN behaviour of SparseSolverNUM.cpp:194-203) per block
template <int B>
__global__ void k_final(int dim, const double* __restrict__ D, const double* __restrict__ Di,
                        const double* __restrict__ v, double* __restrict__ x,
                        double* __restrict__ part) {
  __shared__ double red[8];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  double res = 0.;
  if (r < dim) {
    if (B == 1) {
      const double xn = (1. / D[r]) * v[r];
      const double q = fabs(x[r] - xn) / x[r];
      res = (res < q) ? q : res;
      x[r] = xn;
    } else {
      double t[4];
      mv4(Di + 16 * (size_t)r, v + 4 * (size_t)r, t);
      for (int j = 0; j < 4; ++j) x[4 * (size_t)r + j] = t[j];
    }
  }
  if (B == 1) {
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_xor_sync(0xffffffffu, res, o);
      res = (res < w) ? w : res;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = res;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = red[0];
      for (int i = 1; i < (int)(blockDim.x >> 5); ++i) m = (m < red[i]) ? red[i] : m;
      part[blockIdx.x] = m;
    }
  }
}

template <int B>
__global__ void k_invert_blocks(int dim, const double* __restrict__ D, double* __restrict__ Di) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < dim) inv4(D + 16 * (size_t)r, Di + 16 * (size_t)r);
}

// ---- host-side structure -----------------------------------------------------
struct Csr {
  std::vector<int> ptr, col;
  std::vector<double> val;
};

}  // namespace

struct mst_lu {
  int block = 1, dim = 0;
  int n_fwd_levels = 0, n_bwd_levels = 0;
  std::vector<int> fwd_ptr, bwd_ptr;  // level ranges into the row lists (host)
  // device
  cudaStream_t stream = nullptr;
  double *D = nullptr, *Di = nullptr;
  int *l_ptr = nullptr, *l_col = nullptr, *ua_ptr = nullptr, *ua_col = nullptr,
      *ud_ptr = nullptr, *ud_col = nullptr, *fwd_rows = nullptr, *bwd_rows = nullptr;
  double *l_val = nullptr, *ua_val = nullptr, *ud_val = nullptr;
  double *b = nullptr, *x = nullptr, *t1 = nullptr, *rhs = nullptr, *rhs1 = nullptr,
         *part = nullptr;
  std::vector<void*> allocs;
};

namespace {

mst_status lu_fail(mst_status s, const std::string& m) { return mst_internal_fail(s, m); }

#define LU_CU(call)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return lu_fail(MST_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// rows' entries below (lower) or above the diagonal, sorted by column
// (ascending or descending) and then insertion order
Csr build_rows(int dim, int n, const int* rows, const int* cols, const double* vals, int B,
               bool lower, bool desc) {
  std::vector<int> idx;
  for (int i = 0; i < n; ++i)
    if (lower ? rows[i] > cols[i] : rows[i] < cols[i]) idx.push_back(i);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
    if (rows[a] != rows[b]) return rows[a] < rows[b];
    if (cols[a] != cols[b]) return desc ? cols[a] > cols[b] : cols[a] < cols[b];
    return a < b;
  });
  Csr c;
  c.ptr.assign(dim + 1, 0);
  for (int i : idx) c.ptr[rows[i] + 1]++;
  for (int r = 0; r < dim; ++r) c.ptr[r + 1] += c.ptr[r];
  for (int i : idx) {
    c.col.push_back(cols[i]);
    for (int k = 0; k < B * B; ++k) c.val.push_back(vals[(size_t)B * B * i + k]);
  }
  return c;
}

// rows grouped by level; level(r) = 1 + max level of the rows it reads
void levels(const Csr& c, int dim, bool forward, std::vector<int>* rows_by_level,
            std::vector<int>* ptr, int* n_levels) {
  std::vector<int> lev(dim, 0);
  int maxl = -1;
  for (int t = 0; t < dim; ++t) {
    const int r = forward ? t : dim - 1 - t;
    int l = 0;
    for (int k = c.ptr[r]; k < c.ptr[r + 1]; ++k) l = std::max(l, lev[c.col[k]] + 1);
    lev[r] = l;
    maxl = std::max(maxl, l);
  }
  *n_levels = maxl + 1;
  ptr->assign(maxl + 2, 0);
  for (int r = 0; r < dim; ++r) (*ptr)[lev[r] + 1]++;
  for (int l = 0; l <= maxl; ++l) (*ptr)[l + 1] += (*ptr)[l];
  rows_by_level->assign(dim, 0);
  std::vector<int> fill(ptr->begin(), ptr->end() - 1);
  for (int r = 0; r < dim; ++r) (*rows_by_level)[fill[lev[r]]++] = r;
}

template <class T>
cudaError_t up(mst_lu* s, T** dst, const std::vector<T>& v) {
  const size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void**)dst, bytes);
  if (e != cudaSuccess) return e;
  s->allocs.push_back(*dst);
  if (!v.empty()) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

template <int B>
mst_status lu_iterate(mst_lu* s, int gs, int* iterations) {
  const int dim = s->dim, nb = (dim + 127) / 128;
  int it = 0;
  std::vector<double> part(nb);
  for (it = 0; it < kLuInterval; ++it) {
    if (!gs) {
      k_upper_product<B><<<nb, 128, 0, s->stream>>>(dim, s->ua_ptr, s->ua_col, s->ua_val, s->x,
                                                    s->D, s->Di, s->b, s->t1, 0);
      k_lower_product<B><<<nb, 128, 0, s->stream>>>(dim, s->l_ptr, s->l_col, s->l_val, s->t1,
                                                    s->b, s->rhs);
    } else {
      k_upper_product<B><<<nb, 128, 0, s->stream>>>(dim, s->ua_ptr, s->ua_col, s->ua_val, s->x,
                                                    s->D, s->Di, s->b, s->rhs, 1);
    }
    for (int l = 0; l < s->n_fwd_levels; ++l) {
      const int a = s->fwd_ptr[l], n = s->fwd_ptr[l + 1] - a;
      k_sweep_level<B><<<(n + 127) / 128, 128, 0, s->stream>>>(
          n, s->fwd_rows + a, s->l_ptr, s->l_col, s->l_val, s->D, s->Di, s->rhs);
    }
    const double* last = s->rhs;
    if (!gs) {
      k_middle<B><<<nb, 128, 0, s->stream>>>(dim, s->D, s->Di, s->rhs, s->rhs1);
      for (int l = 0; l < s->n_bwd_levels; ++l) {
        const int a = s->bwd_ptr[l], n = s->bwd_ptr[l + 1] - a;
        k_sweep_level<B><<<(n + 127) / 128, 128, 0, s->stream>>>(
            n, s->bwd_rows + a, s->ud_ptr, s->ud_col, s->ud_val, s->D, s->Di, s->rhs1);
      }
      last = s->rhs1;
    }
    k_final<B><<<nb, 128, 0, s->stream>>>(dim, s->D, s->Di, last, s->x, s->part);
    LU_CU(cudaGetLastError());
    if (B == 1) {
      // the reference's exit test (SparseSolverNUM.cpp:205, :245)
      LU_CU(cudaMemcpyAsync(part.data(), s->part, nb * sizeof(double), cudaMemcpyDeviceToHost,
                            s->stream));
      LU_CU(cudaStreamSynchronize(s->stream));
      double res = 0.;
      for (double p : part) res = (res < p) ? p : res;
      if (res > 1e-10 * 1e-10 && res < 1e-7) {
        ++it;
        break;
      }
    }
  }
  LU_CU(cudaStreamSynchronize(s->stream));
  if (iterations) *iterations = it;
  return MST_OK;
}

}  // namespace

extern "C" {

mst_status mst_lu_create(int block, int dim, int n, const int* rows, const int* cols,
                         const int* ops, const double* vals, mst_lu** out) {
  if (!out || dim <= 0 || n < 0 || (n > 0 && (!rows || !cols || !vals)))
    return lu_fail(MST_EINVAL, "bad arguments");
  if (block != 1 && block != 4) return lu_fail(MST_EINVAL, "block must be 1 or 4");
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (rows[i] < 0 || rows[i] >= dim || cols[i] < 0 || cols[i] >= dim)
      return lu_fail(MST_EINVAL, "entry outside the matrix");
  auto s = new (std::nothrow) mst_lu;
  if (!s) return lu_fail(MST_ENOMEM, "host allocation failed");
  s->block = block;
  s->dim = dim;
  const int BB = block * block;
  // diagonal: setELE sets, addELE adds (scalar); setD sets (blocks)
  std::vector<double> D((size_t)dim * BB, 0.0);
  for (int i = 0; i < n; ++i)
    if (rows[i] == cols[i]) {
      double* d = D.data() + (size_t)BB * rows[i];
      const double* v = vals + (size_t)BB * i;
      if (block == 1 && ops && ops[i] == 1) d[0] += v[0];
      else std::memcpy(d, v, BB * sizeof(double));
    }
  Csr L = build_rows(dim, n, rows, cols, vals, block, true, false);
  Csr Ua = build_rows(dim, n, rows, cols, vals, block, false, false);
  Csr Ud = build_rows(dim, n, rows, cols, vals, block, false, true);
  std::vector<int> fr, br;
  levels(L, dim, true, &fr, &s->fwd_ptr, &s->n_fwd_levels);
  levels(Ud, dim, false, &br, &s->bwd_ptr, &s->n_bwd_levels);
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = up(s, &s->D, D);
  if (e == cudaSuccess) e = up(s, &s->l_ptr, L.ptr);
  if (e == cudaSuccess) e = up(s, &s->l_col, L.col);
  if (e == cudaSuccess) e = up(s, &s->l_val, L.val);
  if (e == cudaSuccess) e = up(s, &s->ua_ptr, Ua.ptr);
  if (e == cudaSuccess) e = up(s, &s->ua_col, Ua.col);
  if (e == cudaSuccess) e = up(s, &s->ua_val, Ua.val);
  if (e == cudaSuccess) e = up(s, &s->ud_ptr, Ud.ptr);
  if (e == cudaSuccess) e = up(s, &s->ud_col, Ud.col);
  if (e == cudaSuccess) e = up(s, &s->ud_val, Ud.val);
  if (e == cudaSuccess) e = up(s, &s->fwd_rows, fr);
  if (e == cudaSuccess) e = up(s, &s->bwd_rows, br);
  const std::vector<double> zero((size_t)dim * block, 0.0);
  for (double** p : {&s->b, &s->x, &s->t1, &s->rhs, &s->rhs1})
    if (e == cudaSuccess) e = up(s, p, zero);
  if (e == cudaSuccess) e = up(s, &s->part, std::vector<double>((dim + 127) / 128 + 1, 0.0));
  if (e == cudaSuccess && block == 4) {
    e = up(s, &s->Di, std::vector<double>((size_t)dim * 16, 0.0));
    // D^-1 once: the reference re-inverts D[i] at every use, always to the
    // same result
    if (e == cudaSuccess) {
      k_invert_blocks<4><<<(dim + 127) / 128, 128, 0, s->stream>>>(dim, s->D, s->Di);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  }
  if (e != cudaSuccess) {
    mst_lu_destroy(s);
    return lu_fail(MST_ECUDA, std::string("mst_lu_create: ") + cudaGetErrorString(e));
  }
  *out = s;
  return MST_OK;
}

mst_status mst_lu_solve(mst_lu* s, int method, const double* b, double* x, int* iterations) {
  if (!s || !b || !x) return lu_fail(MST_EINVAL, "NULL argument");
  if (method != MST_LU_ILUSGS && method != MST_LU_GS)
    return lu_fail(MST_EINVAL, "unknown method");
  if (s->block == 4 && method == MST_LU_GS)
    return lu_fail(MST_EUNSUPPORTED, "the block solver's GS is empty in the reference");
  const size_t bytes = (size_t)s->dim * s->block * sizeof(double);
  LU_CU(cudaMemcpyAsync(s->b, b, bytes, cudaMemcpyHostToDevice, s->stream));
  LU_CU(cudaMemcpyAsync(s->x, x, bytes, cudaMemcpyHostToDevice, s->stream));
  mst_status st = (s->block == 1) ? lu_iterate<1>(s, method == MST_LU_GS, iterations)
                                  : lu_iterate<4>(s, 0, iterations);
  if (st) return st;
  LU_CU(cudaMemcpyAsync(x, s->x, bytes, cudaMemcpyDeviceToHost, s->stream));
  LU_CU(cudaStreamSynchronize(s->stream));
  return MST_OK;
}

mst_status mst_lu_levels(const mst_lu* s, int* forward, int* backward) {
  if (!s) return lu_fail(MST_EINVAL, "NULL argument");
  if (forward) *forward = s->n_fwd_levels;
  if (backward) *backward = s->n_bwd_levels;
  return MST_OK;
}

mst_status mst_lu_destroy(mst_lu* s) {
  if (!s) return MST_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (void* p : s->allocs) cudaFree(p);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return MST_OK;
}

}  // extern "C"
