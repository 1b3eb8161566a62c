// The learned initial field: a message-passing network over the cell
// adjacency whose dense layers run on the tensor cores (tc_gemm.cuh).
// This file holds the GEMM launcher and its C-ABI check entry point.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "ctx.hpp"
#include "tc_gemm.cuh"
#include "tc_gemm_tma.cuh"

namespace mst {
namespace tc {

// Descriptor strides of the no-swizzle K-major layout of k_gemm_bf16's
// tiles: core matrices adjacent along K are 128 bytes apart (leading
// dimension), 8-row groups 1024 bytes apart (stride dimension).
constexpr uint32_t kLBO = 128, kSBO = 1024;

// polls of the GEMM's bounded mbarrier waits (mst_set_wait_limit)
std::atomic<long long> g_wait_limit{-1};

// cuTensorMapEncodeTiled, through the runtime's driver entry point (no
// link-time dependency on the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// tensor map of a row-major [rows][K] BF16 matrix in 128-row x 64-K boxes,
// 128-byte swizzle; rows beyond the matrix read as zeros
bool bf16_tile_map(CUtensorMap* map, const void* base, int rows, int K) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)kBM};
  const cuuint32_t es[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
            box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

// The persistent TMA kernel where it applies (whole K per CTA, K <= 256 in
// tiles of 64, 16-byte-aligned operands; fewer than 128 outputs use one
// 128-wide tile whose missing rows of B the copy fills with zeros); false:
// the caller launches k_gemm_bf16 instead
bool gemm_tma(const GemmArgs& a, cudaStream_t s, cudaError_t* err) {
  *err = cudaSuccess;
  if (a.k_chunk > 0 || a.K % kBK != 0 || a.K / kBK > kTmaMaxKT || a.M <= 0 || a.N <= 0 ||
      (reinterpret_cast<uintptr_t>(a.A) & 15) || (reinterpret_cast<uintptr_t>(a.B) & 15))
    return false;
  CUtensorMap ma, mb;
  if (!bf16_tile_map(&ma, a.A, a.M, a.K) || !bf16_tile_map(&mb, a.B, a.N, a.K)) return false;
  static std::atomic<uint64_t> attr_done{0};
  const int kt = a.K / kBK;
  *err = ensure_smem_limit(k_gemm_tma, tma_smem_bytes(kTmaMaxKT), attr_done);
  if (*err != cudaSuccess) return true;
  // resident CTAs of the device (SMs x CTAs per SM at this K), per K
  static std::atomic<int> resident[kTmaMaxKT + 1];
  int slots = resident[kt].load(std::memory_order_relaxed);
  if (slots <= 0) {
    int dev = 0, sms = 0, per_sm = 0;
    if ((*err = cudaGetDevice(&dev)) != cudaSuccess ||
        (*err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) !=
            cudaSuccess ||
        (*err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_tma, kTmaThreads,
                                                              tma_smem_bytes(kt))) != cudaSuccess)
      return true;
    slots = std::max(1, sms * per_sm);
    resident[kt].store(slots, std::memory_order_relaxed);
  }
  TmaGemm t;
  t.g = a;
  t.kt = kt;
  t.n_ntiles = (a.N + kBN - 1) / kBN;
  t.m_tiles = (a.M + kBM - 1) / kBM;
  // one wave of resident CTAs, each column block with the same number
  int grid = std::min(slots, t.n_ntiles * t.m_tiles);
  grid = std::max(t.n_ntiles, grid / t.n_ntiles * t.n_ntiles);
  k_gemm_tma<<<grid, kTmaThreads, tma_smem_bytes(kt), s>>>(ma, mb, t);
  *err = cudaGetLastError();
  return true;
}

// The split-K TMA kernel where it applies (K and the chunk in tiles of 64,
// 16-byte-aligned operands); false: the caller launches k_gemm_bf16
bool gemm_tma_split(const GemmArgs& a, cudaStream_t s, cudaError_t* err) {
  *err = cudaSuccess;
  if (a.k_chunk <= 0 || a.k_chunk % kBK != 0 || a.K % kBK != 0 || a.M <= 0 || a.N <= 0 ||
      (reinterpret_cast<uintptr_t>(a.A) & 15) || (reinterpret_cast<uintptr_t>(a.B) & 15))
    return false;
  CUtensorMap ma, mb;
  if (!bf16_tile_map(&ma, a.A, a.M, a.K) || !bf16_tile_map(&mb, a.B, a.N, a.K)) return false;
  static std::atomic<uint64_t> attr_done{0};
  *err = ensure_smem_limit(k_gemm_tma_split, split_smem_bytes(), attr_done);
  if (*err != cudaSuccess) return true;
  const dim3 grid((a.M + kBM - 1) / kBM, (a.N + kBN - 1) / kBN, (a.K + a.k_chunk - 1) / a.k_chunk);
  k_gemm_tma_split<<<grid, kSplitThreads, split_smem_bytes(), s>>>(ma, mb, a);
  *err = cudaGetLastError();
  return true;
}

cudaError_t gemm(const GemmArgs& a0, cudaStream_t s) {
  static std::atomic<uint64_t> attr_done{0}, attr_done16{0};
  const bool narrow = a0.N <= 16;
  cudaError_t e = narrow ? ensure_smem_limit(k_gemm_bf16<16>, smem_bytes<16>(), attr_done16)
                         : ensure_smem_limit(k_gemm_bf16<kBN>, kSmemBytes, attr_done);
  if (e != cudaSuccess) return e;
  GemmArgs a = a0;
  const long long lim = g_wait_limit.load(std::memory_order_relaxed);
  a.spin_limit = lim < 0 ? kSpinLimit : (unsigned)std::min<long long>(lim, 0xFFFFFFFFll);
  // MSTCFD_GEMM_TMA=0 keeps every GEMM on k_gemm_bf16 (for comparisons)
  static const bool use_tma = [] {
    const char* v = std::getenv("MSTCFD_GEMM_TMA");
    return !v || std::atoi(v) != 0;
  }();
  if (a.lbo == 0 && use_tma) {
    cudaError_t te;
    if (a.k_chunk > 0 ? gemm_tma_split(a, s, &te) : gemm_tma(a, s, &te)) return te;
  }
  if (a.lbo == 0) {
    a.lbo = kLBO;
    a.sbo = kSBO;
  }
  const int splits = a.k_chunk > 0 ? (a.K + a.k_chunk - 1) / a.k_chunk : 1;
  if (narrow) {
    dim3 grid((a.M + kBM - 1) / kBM, 1, splits);
    k_gemm_bf16<16><<<grid, kGemmThreads, smem_bytes<16>(), s>>>(a);
    return cudaGetLastError();
  }
  dim3 grid((a.M + kBM - 1) / kBM, (a.N + kBN - 1) / kBN, splits);
  k_gemm_bf16<kBN><<<grid, kGemmThreads, kSmemBytes, s>>>(a);
  return cudaGetLastError();
}

// C[M][N] = sum over z of part[z][M][N], in z order (deterministic)
__global__ void k_reduce_splits(const float* __restrict__ part, int splits, size_t mn,
                                float* __restrict__ c) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= mn) return;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * mn + i];
  c[i] = s;
}

}  // namespace tc
}  // namespace mst

// ---------------------------------------------------------------------------
// The network.  Per cell c of a mesh graph (interior-face neighbours N(c)):
//   h0 = relu(We x + be)                                 x: 16 features (K 64)
//   h_{l+1} = h_l + relu(Wl [h_l, mean_{j in N(c)} h_j] + bl),  l = 0..2
//   y = Wd h3 + bd                                       4 outputs
// Width 128.  GEMM operands are BF16 (weights and activations rounded once
// per use), accumulation and the residual stream FP32; master weights and
// Adam moments FP32.  Training minimises the mean squared error of y.
// ---------------------------------------------------------------------------
namespace {

constexpr int kW = 128;       // hidden width
constexpr int kIn = 16;       // input features
constexpr int kInK = 64;      // padded K of the first layer
constexpr int kOut = 4;
constexpr int kLayers = 3;
constexpr int kZ = 2 * kW;    // [h, mean of neighbours]
constexpr int kMaxSplits = 320;  // split-K CTAs of a weight-gradient GEMM

__global__ void k_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// Z = [bf16(h_c), bf16(mean_{j in N(c)} h_j)] (rows >= n: zero); one warp
// per cell, each lane four features (16-byte loads, 8-byte stores), the
// neighbours summed in list order
constexpr int kCellsPerBlock = 8;
__device__ __forceinline__ uint2 bf16x4(float4 v) {
  const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y), b = __floats2bfloat162_rn(v.z, v.w);
  return make_uint2(*reinterpret_cast<const uint32_t*>(&a), *reinterpret_cast<const uint32_t*>(&b));
}
__global__ void __launch_bounds__(32 * kCellsPerBlock)
    k_build_z(const float* __restrict__ h, const int* __restrict__ ptr,
              const int* __restrict__ nbr, int n, int n_pad, __nv_bfloat16* __restrict__ z) {
  const int c = blockIdx.x * kCellsPerBlock + (threadIdx.x >> 5), k = (threadIdx.x & 31) * 4;
  if (c >= n_pad) return;
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f), hc = a;
  if (c < n) {
    hc = *reinterpret_cast<const float4*>(h + (size_t)c * kW + k);
    const int b = ptr[c], e = ptr[c + 1];
    for (int i = b; i < e; ++i) {
      const float4 v = *reinterpret_cast<const float4*>(h + (size_t)nbr[i] * kW + k);
      a.x += v.x;
      a.y += v.y;
      a.z += v.z;
      a.w += v.w;
    }
    if (e > b) {
      const float d = (float)(e - b);
      a.x /= d;
      a.y /= d;
      a.z /= d;
      a.w /= d;
    }
  }
  *reinterpret_cast<uint2*>(z + (size_t)c * kZ + k) = bf16x4(hc);
  *reinterpret_cast<uint2*>(z + (size_t)c * kZ + kW + k) = bf16x4(a);
}

// dst[w][n_pad] = transpose of src[n][w] (BF16), zero for rows >= n
__global__ void k_transpose_bf16(const __nv_bfloat16* __restrict__ src, int n, int w,
                                 int n_pad, __nv_bfloat16* __restrict__ dst) {
  __shared__ __nv_bfloat16 t[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    t[i][threadIdx.x] = (r < n && c < w) ? src[(size_t)r * w + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (c < w && r < n_pad) dst[(size_t)c * n_pad + r] = t[threadIdx.x][i];
  }
}

// loss and dY = 2 (y - t) / (n * kOut); per-block partial losses
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, int n,
                      float* __restrict__ dy, double* __restrict__ part) {
  __shared__ double red[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (i < n * kOut) {
    const float d = y[i] - t[i];
    dy[i] = 2.f * d / (float)(n * kOut);
    l = (double)d * d;
  }
  red[threadIdx.x] = l;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// dP = dH (.) [r > 0] with r = h_next - h_prev (the relu output), FP32 and a
// BF16 copy; pad rows zero
__global__ void k_relu_back(const float* __restrict__ dh, const float* __restrict__ hn,
                            const float* __restrict__ hp, int n, int n_pad,
                            float* __restrict__ dp, __nv_bfloat16* __restrict__ dpb) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)n_pad * kW) return;
  float v = 0.f;
  if (i < (size_t)n * kW) {
    const float r = hp ? hn[i] - hp[i] : hn[i];
    v = r > 0.f ? dh[i] : 0.f;
  }
  dp[i] = v;
  dpb[i] = __float2bfloat16_rn(v);
}

// dH_l = dH_{l+1} + dZ[:, :kW] + sum_{c in N(j)} dZ[c, kW:] / |N(c)|; one
// warp per cell, each lane four features, the neighbours in list order
__global__ void __launch_bounds__(32 * kCellsPerBlock)
    k_agg_back(const float* __restrict__ dhn, const float* __restrict__ dz,
               const int* __restrict__ ptr, const int* __restrict__ nbr, int n,
               float* __restrict__ dh) {
  const int j = blockIdx.x * kCellsPerBlock + (threadIdx.x >> 5), k = (threadIdx.x & 31) * 4;
  if (j >= n) return;
  const float4 x = *reinterpret_cast<const float4*>(dhn + (size_t)j * kW + k);
  const float4 y = *reinterpret_cast<const float4*>(dz + (size_t)j * kZ + k);
  float4 v = make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
  for (int i = ptr[j]; i < ptr[j + 1]; ++i) {
    const int c = nbr[i];
    const float deg = (float)(ptr[c + 1] - ptr[c]);
    const float4 u = *reinterpret_cast<const float4*>(dz + (size_t)c * kZ + kW + k);
    v.x += u.x / deg;
    v.y += u.y / deg;
    v.z += u.z / deg;
    v.w += u.w / deg;
  }
  *reinterpret_cast<float4*>(dh + (size_t)j * kW + k) = v;
}

// Column sums of g[n][w] (bias gradients), w dividing 256, in a fixed order
// (deterministic): block b sums rows [b*chunk, (b+1)*chunk), its 256 threads
// reading whole rows (thread t: column t % w, row offset t / w), into
// part[b][w]; k_colsum_parts then adds the blocks' partials in block order.
__global__ void __launch_bounds__(256) k_colsum(const float* __restrict__ g, int n, int w,
                                                int chunk, float* __restrict__ part) {
  __shared__ float red[256];
  const int t = threadIdx.x, col = t % w, rows = 256 / w;
  const int r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  float s = 0.f;
  for (int r = r0 + t / w; r < r1; r += rows) s += g[(size_t)r * w + col];
  red[t] = s;
  __syncthreads();
  if (t < w) {
    float acc = red[t];
    for (int k = 1; k < rows; ++k) acc += red[t + k * w];
    part[(size_t)blockIdx.x * w + t] = acc;
  }
}
__global__ void k_colsum_parts(const float* __restrict__ part, int blocks, int w,
                               float* __restrict__ out) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= w) return;
  float acc = 0.f;
  for (int b = 0; b < blocks; ++b) acc += part[(size_t)b * w + col];
  out[col] = acc;
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float c1,
                       float c2, __nv_bfloat16* __restrict__ wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float x = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
  w[i] = x;
  if (wb) wb[i] = __float2bfloat16_rn(x);
}

}  // namespace

// One parameter tensor: FP32 master, BF16 copy (GEMM operand), gradient,
// Adam moments.  Weights are [rows = outputs][cols = inputs], the B
// operand layout of the GEMM.
struct MpnnParam {
  int rows = 0, cols = 0;
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16* wb = nullptr;
  int size() const { return rows * cols; }
};

struct mst_mpnn {
  MpnnParam W[2 * (kLayers + 2)];  // We, be, Wl0, bl0, ..., Wd, bd
  int step = 0;
  // work buffers for up to cap cells
  int cap = 0;
  int* err = nullptr;
  double* lpart = nullptr;
  std::vector<void*> bufs;
  float* H[kLayers + 1] = {};      // FP32 residual stream
  __nv_bfloat16 *X = nullptr, *Z[kLayers] = {}, *Hb = nullptr;
  float *Y = nullptr, *T = nullptr, *dY = nullptr, *dH = nullptr, *dHn = nullptr,
        *dP = nullptr, *dZ = nullptr;
  __nv_bfloat16 *dPb = nullptr, *tA = nullptr, *tB = nullptr, *dYb = nullptr, *WdT = nullptr,
                *WlT = nullptr;
  float* part = nullptr;  // split-K partial products of the weight gradients
  float* feat = nullptr;  // the graph's FP32 features [cap][16]
  int *ptr = nullptr, *nbr = nullptr;
  int n_nbr_cap = 0;
  int n = 0;  // cells of the current graph
  // live timing of the tensor-core GEMM launches (mst_mpnn_profile): one
  // event pair per launch on the network's stream, with the launch's
  // 2MNK flops and its operand/result bytes
  struct GemmRec {
    cudaEvent_t a = nullptr, b = nullptr;
    double flops = 0.0, bytes = 0.0;
  };
  bool prof = false;
  std::vector<GemmRec> recs;
  size_t n_recs = 0;
};

namespace {

MpnnParam& P(mst_mpnn* m, int i) { return m->W[i]; }
enum { kWe = 0, kBe = 1, kWd = 2 * kLayers + 2, kBd = 2 * kLayers + 3 };
int wl(int l) { return 2 + 2 * l; }
int bl(int l) { return 3 + 2 * l; }

template <class T>
cudaError_t nalloc(mst_mpnn* m, T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T));
  if (e == cudaSuccess) {
    m->bufs.push_back(*p);
    e = cudaMemset(*p, 0, std::max<size_t>(count, 1) * sizeof(T));
  }
  return e;
}

int pad128(int n) { return (n + 127) / 128 * 128; }
int pad64(int n) { return (n + 63) / 64 * 64; }

cudaError_t ensure_cap(mst_mpnn* m, int n, int n_nbr) {
  cudaError_t e = cudaSuccess;
  if (n_nbr > m->n_nbr_cap) {
    if (m->nbr) cudaFree(m->nbr);
    e = cudaMalloc(&m->nbr, sizeof(int) * (size_t)n_nbr);
    m->n_nbr_cap = n_nbr;
  }
  if (e != cudaSuccess || n <= m->cap) return e;
  // grow: free the old work buffers (parameters live in m->W)
  for (void* p : m->bufs) cudaFree(p);
  m->bufs.clear();
  const int np = pad128(n), nk = pad64(n);
  m->cap = n;
  for (int l = 0; l <= kLayers && e == cudaSuccess; ++l) e = nalloc(m, &m->H[l], (size_t)np * kW);
  for (int l = 0; l < kLayers && e == cudaSuccess; ++l) e = nalloc(m, &m->Z[l], (size_t)np * kZ);
  if (e == cudaSuccess) e = nalloc(m, &m->X, (size_t)np * kInK);
  if (e == cudaSuccess) e = nalloc(m, &m->Hb, (size_t)np * kW);
  if (e == cudaSuccess) e = nalloc(m, &m->Y, (size_t)np * kOut);
  if (e == cudaSuccess) e = nalloc(m, &m->T, (size_t)np * kOut);
  if (e == cudaSuccess) e = nalloc(m, &m->dY, (size_t)np * kOut);
  if (e == cudaSuccess) e = nalloc(m, &m->dYb, (size_t)np * kInK);
  if (e == cudaSuccess) e = nalloc(m, &m->dH, (size_t)np * kW);
  if (e == cudaSuccess) e = nalloc(m, &m->dHn, (size_t)np * kW);
  if (e == cudaSuccess) e = nalloc(m, &m->dP, (size_t)np * kW);
  if (e == cudaSuccess) e = nalloc(m, &m->dPb, (size_t)np * kW);
  if (e == cudaSuccess) e = nalloc(m, &m->dZ, (size_t)np * kZ);
  if (e == cudaSuccess) e = nalloc(m, &m->tA, (size_t)kZ * nk);
  if (e == cudaSuccess) e = nalloc(m, &m->tB, (size_t)kZ * nk);
  if (e == cudaSuccess) e = nalloc(m, &m->ptr, (size_t)n + 1);
  if (e == cudaSuccess) e = nalloc(m, &m->lpart, (size_t)(np * kOut + 255) / 256 + 1);
  if (e == cudaSuccess) e = nalloc(m, &m->err, 1);
  if (e == cudaSuccess) e = nalloc(m, &m->WdT, (size_t)kW * kInK);
  if (e == cudaSuccess) e = nalloc(m, &m->WlT, (size_t)kZ * kW);
  if (e == cudaSuccess) e = nalloc(m, &m->part, (size_t)kMaxSplits * kW * kZ);
  if (e == cudaSuccess) e = nalloc(m, &m->feat, (size_t)n * kIn);
  return e;
}

// brackets one GEMM launch with an event pair when profiling is on
struct GemmTimer {
  mst_mpnn* m;
  mst_mpnn::GemmRec* r = nullptr;
  GemmTimer(mst_mpnn* mm, double flops, double bytes) : m(mm) {
    if (!m->prof) return;
    if (m->n_recs == m->recs.size()) {
      mst_mpnn::GemmRec g;
      if (cudaEventCreate(&g.a) != cudaSuccess || cudaEventCreate(&g.b) != cudaSuccess) return;
      m->recs.push_back(g);
    }
    r = &m->recs[m->n_recs++];
    r->flops = flops;
    r->bytes = bytes;
    cudaEventRecord(r->a, 0);
  }
  ~GemmTimer() {
    if (r) cudaEventRecord(r->b, 0);
  }
};

cudaError_t gemm(mst_mpnn* m, const __nv_bfloat16* A, const __nv_bfloat16* B, float* C, int M,
                 int N, int K, int ldc, const float* bias, int relu, int acc) {
  GemmTimer timer(m, 2.0 * M * N * K,
                  2.0 * ((double)M * K + (double)N * K) + 4.0 * M * N * (acc ? 2 : 1));
  mst::tc::GemmArgs g{};
  g.A = A;
  g.B = B;
  g.C = C;
  g.bias = bias;
  g.M = M;
  g.N = N;
  g.K = K;
  g.ldc = ldc;
  g.relu = relu;
  g.accumulate_c = acc;
  g.err = m->err;
  return mst::tc::gemm(g, 0);
}

// Weight gradients: M, N small (<= 256), K = the number of cells.  Split K
// over up to kMaxSplits CTAs per output tile, then add the partial products
// in a fixed order.
cudaError_t gemm_wgrad(mst_mpnn* m, const __nv_bfloat16* A, const __nv_bfloat16* B, float* C,
                       int M, int N, int K, int ldc) {
  const int kt = K / mst::tc::kBK;  // K tiles
  // about two CTAs per SM over the output tiles, each with at least 4 K
  // tiles (the SM count read once, thread-safe; it only sizes the split)
  static const int sms = [] {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      n = 148;
    return n;
  }();
  const int n_tiles = ((M + mst::tc::kBM - 1) / mst::tc::kBM) * ((N + mst::tc::kBN - 1) / mst::tc::kBN);
  const int splits =
      std::min(kMaxSplits, std::max(1, std::min(2 * sms / std::max(1, n_tiles), kt / 4)));
  const int chunk = ((kt + splits - 1) / splits) * mst::tc::kBK;
  const int used = (K + chunk - 1) / chunk;
  mst::tc::GemmArgs g{};
  g.A = A;
  g.B = B;
  g.C = m->part;
  g.M = M;
  g.N = N;
  g.K = K;
  g.ldc = ldc;
  g.err = m->err;
  g.k_chunk = chunk;
  cudaError_t e;
  {
    GemmTimer timer(m, 2.0 * M * N * K,
                    2.0 * ((double)M * K + (double)N * K) + 4.0 * used * M * N);
    e = mst::tc::gemm(g, 0);
  }
  if (e != cudaSuccess) return e;
  const size_t mn = (size_t)M * ldc;
  mst::tc::k_reduce_splits<<<(unsigned)((mn + 255) / 256), 256>>>(m->part, used, mn, C);
  return cudaGetLastError();
}

// bias gradient out[w] = column sums of g[n][w], through the split-K
// partial buffer (free between weight-gradient GEMMs)
void colsum(mst_mpnn* m, const float* g, int n, int w, float* out) {
  const int blocks = std::max(1, std::min(296, (n + 255) / 256));
  const int chunk = (n + blocks - 1) / blocks;
  k_colsum<<<blocks, 256>>>(g, n, w, chunk, m->part);
  k_colsum_parts<<<(w + 127) / 128, 128>>>(m->part, blocks, w, out);
}

cudaError_t transpose(const __nv_bfloat16* src, int n, int w, int n_pad, __nv_bfloat16* dst) {
  dim3 grid((n_pad + 31) / 32, (w + 31) / 32), block(32, 8);
  k_transpose_bf16<<<grid, block>>>(src, n, w, n_pad, dst);
  return cudaGetLastError();
}

// forward over the graph loaded in m (n cells); Y = outputs
cudaError_t forward(mst_mpnn* m, int n) {
  const int np = pad128(n);
  cudaError_t e = gemm(m, m->X, P(m, kWe).wb, m->H[0], np, kW, kInK, kW, P(m, kBe).w, 1, 0);
  for (int l = 0; l < kLayers && e == cudaSuccess; ++l) {
    k_build_z<<<(np + kCellsPerBlock - 1) / kCellsPerBlock, 32 * kCellsPerBlock>>>(
        m->H[l], m->ptr, m->nbr, n, np, m->Z[l]);
    e = cudaMemcpyAsync(m->H[l + 1], m->H[l], sizeof(float) * (size_t)np * kW,
                        cudaMemcpyDeviceToDevice, 0);
    if (e == cudaSuccess)
      e = gemm(m, m->Z[l], P(m, wl(l)).wb, m->H[l + 1], np, kW, kZ, kW, P(m, bl(l)).w, 1, 1);
  }
  if (e == cudaSuccess) {
    const size_t cnt = (size_t)np * kW;
    k_to_bf16<<<(unsigned)((cnt + 255) / 256), 256>>>(m->H[kLayers], m->Hb, cnt);
    e = gemm(m, m->Hb, P(m, kWd).wb, m->Y, np, kOut, kW, kOut, P(m, kBd).w, 0, 0);
  }
  return e == cudaSuccess ? cudaGetLastError() : e;
}

// backward of the mean squared error against m->T; gradients into W[].g;
// returns the loss through *loss
cudaError_t backward(mst_mpnn* m, int n, double* loss) {
  const int np = pad128(n), nk = pad64(n);
  const int nb = (n * kOut + 255) / 256;
  k_mse<<<nb, 256>>>(m->Y, m->T, n, m->dY, m->lpart);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  std::vector<double> part(nb);
  e = cudaMemcpy(part.data(), m->lpart, sizeof(double) * nb, cudaMemcpyDeviceToHost);
  double l = 0.0;
  for (double x : part) l += x;
  *loss = l / (double)(n * kOut);
  // decoder: dWd = dY^T H3, dbd = colsum dY, dH3 = dY Wd.  dY as BF16:
  // compact [n][4] (in dPb) for the transpose, and widened to a [np][64]
  // A operand (columns >= 4 zero) for dH3
  e = cudaMemset(m->dYb, 0, sizeof(__nv_bfloat16) * (size_t)np * kInK);
  if (e != cudaSuccess) return e;
  {
    const size_t cnt = (size_t)n * kOut;
    k_to_bf16<<<(unsigned)((cnt + 255) / 256), 256>>>(m->dY, m->dPb, cnt);
    e = cudaMemcpy2DAsync(m->dYb, kInK * sizeof(__nv_bfloat16), m->dPb,
                          kOut * sizeof(__nv_bfloat16), kOut * sizeof(__nv_bfloat16), n,
                          cudaMemcpyDeviceToDevice, 0);
    if (e != cudaSuccess) return e;
  }
  e = transpose(m->dPb, n, kOut, nk, m->tA);  // dY^T [4][nk]
  if (e == cudaSuccess) e = transpose(m->Hb, n, kW, nk, m->tB);  // H3^T [128][nk]
  if (e == cudaSuccess)
    e = gemm_wgrad(m, m->tA, m->tB, P(m, kWd).g, kOut, kW, nk, kW);
  if (e != cudaSuccess) return e;
  colsum(m, m->dY, n, kOut, P(m, kBd).g);
  // dH3 = dY . Wd : B operand = Wd^T [128][64] (K = 4 padded with zeros)
  e = transpose(P(m, kWd).wb, kOut, kW, kInK, m->WdT);
  if (e == cudaSuccess) e = gemm(m, m->dYb, m->WdT, m->dH, np, kW, kInK, kW, nullptr, 0, 0);
  for (int l = kLayers - 1; l >= 0 && e == cudaSuccess; --l) {
    // dP = dH_{l+1} (.) relu'
    const size_t cnt = (size_t)np * kW;
    k_relu_back<<<(unsigned)((cnt + 255) / 256), 256>>>(m->dH, m->H[l + 1], m->H[l], n, np,
                                                         m->dP, m->dPb);
    e = transpose(m->dPb, n, kW, nk, m->tA);            // dP^T [128][nk]
    if (e == cudaSuccess) e = transpose(m->Z[l], n, kZ, nk, m->tB);  // Z^T [256][nk]
    if (e == cudaSuccess)
      e = gemm_wgrad(m, m->tA, m->tB, P(m, wl(l)).g, kW, kZ, nk, kZ);
    if (e != cudaSuccess) break;
    colsum(m, m->dP, n, kW, P(m, bl(l)).g);
    // dZ = dP . Wl : B operand = Wl^T [256][128]
    e = transpose(P(m, wl(l)).wb, kW, kZ, kW, m->WlT);
    if (e == cudaSuccess) e = gemm(m, m->dPb, m->WlT, m->dZ, np, kZ, kW, kZ, nullptr, 0, 0);
    if (e != cudaSuccess) break;
    std::swap(m->dH, m->dHn);  // dHn = dH_{l+1}
    k_agg_back<<<(n + kCellsPerBlock - 1) / kCellsPerBlock, 32 * kCellsPerBlock>>>(
        m->dHn, m->dZ, m->ptr, m->nbr, n, m->dH);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return e;
  // encoder: dP0 = dH0 (.) [H0 > 0]; dWe = dP0^T X; dbe
  {
    const size_t cnt = (size_t)np * kW;
    k_relu_back<<<(unsigned)((cnt + 255) / 256), 256>>>(m->dH, m->H[0], nullptr, n, np, m->dP,
                                                         m->dPb);
    e = transpose(m->dPb, n, kW, nk, m->tA);
    if (e == cudaSuccess) e = transpose(m->X, n, kInK, nk, m->tB);
    if (e == cudaSuccess)
      e = gemm_wgrad(m, m->tA, m->tB, P(m, kWe).g, kW, kInK, nk, kInK);
    if (e == cudaSuccess) colsum(m, m->dP, n, kW, P(m, kBe).g);
  }
  return e == cudaSuccess ? cudaGetLastError() : e;
}

}  // namespace
namespace {

// features [n][16] FP32 -> X [np][64] BF16 (zero padding)
__global__ void k_features(const float* __restrict__ f, int n, int np,
                           __nv_bfloat16* __restrict__ x) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)np * kInK) return;
  const int r = (int)(i / kInK), c = (int)(i % kInK);
  x[i] = __float2bfloat16_rn((r < n && c < kIn) ? f[(size_t)r * kIn + c] : 0.f);
}

// xorshift64* uniform in [-1, 1)
double urand(uint64_t& s) {
  s ^= s >> 12;
  s ^= s << 25;
  s ^= s >> 27;
  const uint64_t r = s * 2685821657736338717ull;
  return (double)(r >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

}  // namespace

extern "C" {

int mst_mpnn_num_params(void) {
  return kW * kInK + kW + kLayers * (kW * kZ + kW) + kOut * kW + kOut;
}

mst_status mst_mpnn_create(uint64_t seed, mst_mpnn** out) {
  if (!out) return mst_internal_fail(MST_EINVAL, "NULL argument");
  mst_mpnn* m = new mst_mpnn();
  const int shapes[2 * (kLayers + 2)][2] = {{kW, kInK}, {1, kW}, {kW, kZ}, {1, kW}, {kW, kZ},
                                            {1, kW},   {kW, kZ}, {1, kW}, {kOut, kW}, {1, kOut}};
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 2 * (kLayers + 2) && e == cudaSuccess; ++i) {
    MpnnParam& p = m->W[i];
    p.rows = shapes[i][0];
    p.cols = shapes[i][1];
    const size_t n = (size_t)p.size();
    std::vector<float> w(n, 0.f);
    if (p.rows > 1) {
      // Glorot-uniform over the real fan-in (the first layer's is 16)
      const int fan_in = (i == kWe) ? kIn : p.cols;
      const double a = std::sqrt(6.0 / (fan_in + p.rows));
      for (int r = 0; r < p.rows; ++r)
        for (int c = 0; c < p.cols; ++c)
          w[(size_t)r * p.cols + c] = (i == kWe && c >= kIn) ? 0.f : (float)(a * urand(st));
    }
    std::vector<__nv_bfloat16> wb(n);
    for (size_t k = 0; k < n; ++k) wb[k] = __float2bfloat16_rn(w[k]);
    e = cudaMalloc(&p.w, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&p.g, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&p.m, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&p.v, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&p.wb, n * 2);
    if (e == cudaSuccess) e = cudaMemcpy(p.w, w.data(), n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p.wb, wb.data(), n * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(p.g, 0, n * 4);
    if (e == cudaSuccess) e = cudaMemset(p.m, 0, n * 4);
    if (e == cudaSuccess) e = cudaMemset(p.v, 0, n * 4);
  }
  if (e != cudaSuccess) {
    mst_mpnn_destroy(m);
    return mst_internal_fail(MST_ECUDA, std::string("mpnn create: ") + cudaGetErrorString(e));
  }
  *out = m;
  return MST_OK;
}

mst_status mst_mpnn_destroy(mst_mpnn* m) {
  if (!m) return MST_OK;
  cudaDeviceSynchronize();
  for (auto& p : m->W) {
    cudaFree(p.w);
    cudaFree(p.g);
    cudaFree(p.m);
    cudaFree(p.v);
    cudaFree(p.wb);
  }
  for (void* p : m->bufs) cudaFree(p);
  cudaFree(m->nbr);
  for (auto& r : m->recs) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  delete m;
  return MST_OK;
}

mst_status mst_mpnn_profile(mst_mpnn* m, int on) {
  if (!m) return mst_internal_fail(MST_EINVAL, "NULL network");
  m->prof = on != 0;
  m->n_recs = 0;
  return MST_OK;
}

mst_status mst_mpnn_profile_read(mst_mpnn* m, double out[4]) {
  if (!m || !out) return mst_internal_fail(MST_EINVAL, "NULL argument");
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess)
    return mst_internal_fail(MST_ECUDA, std::string("mpnn profile: ") + cudaGetErrorString(e));
  double ms = 0.0, fl = 0.0, by = 0.0;
  for (size_t i = 0; i < m->n_recs; ++i) {
    float t = 0.f;
    e = cudaEventElapsedTime(&t, m->recs[i].a, m->recs[i].b);
    if (e != cudaSuccess)
      return mst_internal_fail(MST_ECUDA, std::string("mpnn profile: ") + cudaGetErrorString(e));
    ms += t;
    fl += m->recs[i].flops;
    by += m->recs[i].bytes;
  }
  out[0] = ms;
  out[1] = fl;
  out[2] = by;
  out[3] = (double)m->n_recs;
  m->n_recs = 0;
  return MST_OK;
}

mst_status mst_mpnn_set_graph(mst_mpnn* m, int n, const float* features, const int* nbr_ptr,
                              const int* nbr) {
  if (!m || n <= 0 || !features || !nbr_ptr || !nbr)
    return mst_internal_fail(MST_EINVAL, "bad graph arguments");
  const int n_nbr = nbr_ptr[n];
  for (int i = 0; i < n; ++i)
    if (nbr_ptr[i + 1] < nbr_ptr[i]) return mst_internal_fail(MST_EINVAL, "nbr_ptr not ascending");
  for (int i = 0; i < n_nbr; ++i)
    if (nbr[i] < 0 || nbr[i] >= n) return mst_internal_fail(MST_EINVAL, "neighbour id out of range");
  cudaError_t e = ensure_cap(m, n, std::max(n_nbr, 1));
  float* df = m->feat;
  if (e == cudaSuccess)
    e = cudaMemcpy(df, features, sizeof(float) * (size_t)n * kIn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(m->ptr, nbr_ptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && n_nbr)
    e = cudaMemcpy(m->nbr, nbr, sizeof(int) * (size_t)n_nbr, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    const int np = pad128(n);
    const size_t cnt = (size_t)np * kInK;
    k_features<<<(unsigned)((cnt + 255) / 256), 256>>>(df, n, np, m->X);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, std::string("mpnn graph: ") + cudaGetErrorString(e));
  m->n = n;
  return MST_OK;
}

mst_status mst_mpnn_set_targets(mst_mpnn* m, const float* t) {
  if (!m || !t || m->n <= 0) return mst_internal_fail(MST_EINVAL, "no graph or NULL targets");
  cudaError_t e = cudaMemcpy(m->T, t, sizeof(float) * (size_t)m->n * kOut, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, cudaGetErrorString(e));
  return MST_OK;
}

mst_status mst_mpnn_forward(mst_mpnn* m, float* y) {
  if (!m || m->n <= 0) return mst_internal_fail(MST_EINVAL, "no graph");
  cudaError_t e = cudaMemset(m->err, 0, sizeof(int));
  if (e == cudaSuccess) e = forward(m, m->n);
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&herr, m->err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && y)
    e = cudaMemcpy(y, m->Y, sizeof(float) * (size_t)m->n * kOut, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, std::string("mpnn forward: ") + cudaGetErrorString(e));
  if (herr == 2)
    return mst_internal_fail(MST_ECUDA, "mpnn forward: shared memory not 1024-byte aligned for TMA");
  if (herr) return mst_internal_fail(MST_ETIMEOUT, "mpnn forward: a tensor-core wait timed out");
  return MST_OK;
}

mst_status mst_mpnn_backward(mst_mpnn* m, double* loss) {
  if (!m || m->n <= 0) return mst_internal_fail(MST_EINVAL, "no graph");
  double l = 0.0;
  cudaError_t e = backward(m, m->n, &l);
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&herr, m->err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, std::string("mpnn backward: ") + cudaGetErrorString(e));
  if (herr == 2)
    return mst_internal_fail(MST_ECUDA, "mpnn backward: shared memory not 1024-byte aligned for TMA");
  if (herr) return mst_internal_fail(MST_ETIMEOUT, "mpnn backward: a tensor-core wait timed out");
  if (loss) *loss = l;
  return MST_OK;
}

// all parameters (which = 0) or gradients (1), in the order We, be, W0, b0,
// W1, b1, W2, b2, Wd, bd, each row-major [outputs][inputs]
mst_status mst_mpnn_get(mst_mpnn* m, int which, float* out) {
  if (!m || !out) return mst_internal_fail(MST_EINVAL, "NULL argument");
  size_t off = 0;
  for (auto& p : m->W) {
    const size_t n = (size_t)p.size();
    cudaError_t e = cudaMemcpy(out + off, which ? p.g : p.w, n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, cudaGetErrorString(e));
    off += n;
  }
  return MST_OK;
}

mst_status mst_mpnn_set_weights(mst_mpnn* m, const float* w) {
  if (!m || !w) return mst_internal_fail(MST_EINVAL, "NULL argument");
  size_t off = 0;
  for (auto& p : m->W) {
    const size_t n = (size_t)p.size();
    std::vector<__nv_bfloat16> wb(n);
    for (size_t k = 0; k < n; ++k) wb[k] = __float2bfloat16_rn(w[off + k]);
    cudaError_t e = cudaMemcpy(p.w, w + off, n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p.wb, wb.data(), n * 2, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, cudaGetErrorString(e));
    off += n;
  }
  return MST_OK;
}

mst_status mst_mpnn_adam_step(mst_mpnn* m, float lr) {
  if (!m) return mst_internal_fail(MST_EINVAL, "NULL network");
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
  for (auto& p : m->W) {
    const int n = p.size();
    k_adam<<<(n + 255) / 256, 256>>>(p.w, p.g, p.m, p.v, n, lr, b1, b2, c1, c2, p.wb);
  }
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, cudaGetErrorString(e));
  return MST_OK;
}


mst_status mst_set_wait_limit(long long polls) {
  mst::tc::g_wait_limit.store(polls < 0 ? -1 : polls, std::memory_order_relaxed);
  return MST_OK;
}

mst_status mst_tc_gemm_check(const uint16_t* A, const uint16_t* B, const float* bias, float* C,
                             int M, int N, int K, int relu, int layout) {
  if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0 || K % mst::tc::kBK != 0)
    return mst_internal_fail(MST_EINVAL, "bad GEMM arguments (K must be a multiple of 64)");
  __nv_bfloat16 *dA = nullptr, *dB = nullptr;
  float *dC = nullptr, *dbias = nullptr;
  int* derr = nullptr;
  auto cleanup = [&]() {
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(dbias);
    cudaFree(derr);
  };
  cudaError_t e = cudaMalloc(&dA, sizeof(uint16_t) * (size_t)M * K);
  if (e == cudaSuccess) e = cudaMalloc(&dB, sizeof(uint16_t) * (size_t)N * K);
  if (e == cudaSuccess) e = cudaMalloc(&dC, sizeof(float) * (size_t)M * N);
  if (e == cudaSuccess && bias) e = cudaMalloc(&dbias, sizeof(float) * N);
  if (e == cudaSuccess) e = cudaMalloc(&derr, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dA, A, sizeof(uint16_t) * (size_t)M * K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, B, sizeof(uint16_t) * (size_t)N * K, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && bias) e = cudaMemcpy(dbias, bias, sizeof(float) * N, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
  if (e == cudaSuccess) {
    mst::tc::GemmArgs g{};
    g.A = dA;
    g.B = dB;
    g.C = dC;
    g.bias = dbias;
    g.M = M;
    g.N = N;
    g.K = K;
    g.ldc = N;
    g.relu = relu;
    g.err = derr;
    if (layout == 1) {  // the other assignment of the two strides
      g.lbo = mst::tc::kSBO;
      g.sbo = mst::tc::kLBO;
    }
    if (layout >= mst::tc::kBK && layout % mst::tc::kBK == 0 && !bias && !relu) {
      // split K in chunks of `layout`, partial products reduced in order
      const int splits = (K + layout - 1) / layout;
      float* part = nullptr;
      e = cudaMalloc(&part, sizeof(float) * (size_t)splits * M * N);
      if (e == cudaSuccess) {
        g.C = part;
        g.k_chunk = layout;
        e = mst::tc::gemm(g, 0);
        const size_t mn = (size_t)M * N;
        if (e == cudaSuccess)
          mst::tc::k_reduce_splits<<<(unsigned)((mn + 255) / 256), 256>>>(part, splits, mn, dC);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        cudaFree(part);
      }
    } else {
      e = mst::tc::gemm(g, 0);
    }
  }
  int herr = 0;
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(C, dC, sizeof(float) * (size_t)M * N, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return mst_internal_fail(MST_ECUDA, std::string("gemm: ") + cudaGetErrorString(e));
  if (herr == 2)
    return mst_internal_fail(MST_ECUDA, "gemm: shared memory not 1024-byte aligned for TMA");
  if (herr) return mst_internal_fail(MST_ETIMEOUT, "gemm: a tensor-core wait timed out");
  return MST_OK;
}

}  // extern "C"
