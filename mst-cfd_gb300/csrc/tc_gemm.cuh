// BF16 tensor-core GEMM on the 5th-generation tensor cores (tcgen05) with
// the accumulator in tensor memory, for the dense layers of the learned
// initial-field network (mpnn.cu) -- the only dense contraction of the
// project.
//
//   C[M, N] (FP32) = A[M, K] (BF16, row-major) . B[N, K]^T (BF16, row-major)
//                    (+ bias[N]) (ReLU) ; optional BF16 copy of C
//
// One CTA of 128 threads per 128 x BN tile (BN = 128, or 16 when N <= 16).  K is walked in
// 64-wide tiles through two shared-memory stages filled with cp.async in
// the canonical no-swizzle K-major layout of the MMA descriptors (8 x 16-
// byte core matrices; core matrices adjacent in K 128 bytes apart, 8-row
// groups 1024 bytes apart).  Thread 0 issues four tcgen05.mma (K = 16 each)
// per tile and commits them to the stage's mbarrier; a stage is refilled
// only after that commit has arrived.  The epilogue reads the accumulator
// with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = rows) and applies
// bias / ReLU.  Every mbarrier wait is bounded (GemmArgs.spin_limit polls;
// mst_set_wait_limit): on timeout the kernel sets *err, waits (bounded by
// the full limit) for its own copies and MMAs, frees its TMEM and returns.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace mst {
namespace tc {

constexpr int kBM = 128, kBN = 128, kBK = 64;
constexpr int kTileA = kBM * kBK * 2;  // bytes
constexpr int kStages = 2;
// output tile width BN: 128, or 16 for narrow outputs (N <= 16; the MMA
// instruction's smallest N at M = 128)
template <int BN>
__host__ __device__ constexpr int tile_b_bytes() { return BN * kBK * 2; }
template <int BN>
__host__ __device__ constexpr int smem_bytes() { return kStages * (kTileA + tile_b_bytes<BN>()) + 64; }
constexpr int kSmemBytes = smem_bytes<kBN>();
// tensor-memory columns allocated for a BN-wide accumulator (a power of two >= 32)
template <int BN>
__host__ __device__ constexpr int tmem_cols() { return BN < 32 ? 32 : BN; }
constexpr unsigned kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) of a [rows x 64] K-major tile
__device__ __forceinline__ uint32_t core_off(int r, int k) {
  return (uint32_t)(((r >> 3) * 8 + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: no swizzle, K-major
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of this architecture
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor of kind::f16: BF16 x BF16 -> FP32, both K-major
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// bounded wait for the phase with the given parity (at most `limit` polls);
// false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          unsigned limit = kSpinLimit) {
  const uint32_t a = smem_u32(bar);
  for (unsigned i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct GemmArgs {
  const __nv_bfloat16* A;  // [M][K]
  const __nv_bfloat16* B;  // [N][K]
  float* C;                // [M][ldc] or nullptr
  __nv_bfloat16* Cb;       // [M][ldcb] BF16 copy or nullptr
  const float* bias;       // [N] or nullptr
  int M, N, K, ldc, ldcb;
  int relu;
  int accumulate_c;        // C += result (FP32 output only)
  uint32_t lbo, sbo;       // descriptor strides (bytes)
  int* err;                // set on a timed-out wait
  unsigned spin_limit;     // polls of each main-loop wait (0: give up at once)
  // split K: CTA z covers K range [z * k_chunk, (z + 1) * k_chunk) and
  // writes its partial product to C + z * M * ldc (no bias / ReLU);
  // k_chunk = 0: one CTA per output tile over the whole K
  int k_chunk;
};

// Epilogue of 16 accumulator columns of one row: bias, ReLU, the residual
// add (accumulate_c) and the stores of C and its BF16 copy (16-byte stores
// where the row allows them; vc / vb: C / Cb rows 16-byte aligned).  prev:
// the 16 values of C already loaded for the residual add (or nullptr).
__device__ __forceinline__ void store16(const GemmArgs& g, bool split, float* Cout, int row,
                                        int n0, int c0, float v[16], bool vc, bool vb,
                                        const float4* prev = nullptr) {
  if (row < g.M && vc && vb && n0 + c0 + 16 <= g.N) {
    const int col0 = n0 + c0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      float x = v[i];
      if (!split && g.bias) x += g.bias[col0 + i];
      if (!split && g.relu) x = fmaxf(x, 0.f);
      v[i] = x;
    }
    if (Cout) {
      float4* p = reinterpret_cast<float4*>(Cout + (size_t)row * g.ldc + col0);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float4 o = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        if (!split && g.accumulate_c) {
          const float4 w = prev ? prev[j] : p[j];
          o.x += w.x;
          o.y += w.y;
          o.z += w.z;
          o.w += w.w;
        }
        p[j] = o;
      }
    }
    if (g.Cb) {
      uint4* pb = reinterpret_cast<uint4*>(g.Cb + (size_t)row * g.ldcb + col0);
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        uint32_t w[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const __nv_bfloat162 b2 = __floats2bfloat162_rn(v[8 * j + 2 * h], v[8 * j + 2 * h + 1]);
          w[h] = *reinterpret_cast<const uint32_t*>(&b2);
        }
        pb[j] = make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
  } else if (row < g.M) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int col = n0 + c0 + i;
      float x = v[i];
      if (!split && g.bias && col < g.N) x += g.bias[col];
      if (!split && g.relu) x = fmaxf(x, 0.f);
      if (col < g.N) {
        if (Cout) {
          float* p = Cout + (size_t)row * g.ldc + col;
          *p = (!split && g.accumulate_c) ? *p + x : x;
        }
        if (g.Cb) g.Cb[(size_t)row * g.ldcb + col] = __float2bfloat16_rn(x);
      }
    }
  }
}

// threads of a CTA; in the epilogue warp w reads TMEM lanes 32 w.. (its
// rows).  (256 threads, with the columns split over two warp groups, measured
// slower: 5.6 against 4.0 ms for the network's 14 GEMMs at batch scale.)
constexpr int kGemmThreads = 128;

template <int BN = kBN>
__global__ void __launch_bounds__(kGemmThreads) k_gemm_bf16(const GemmArgs g) {
  constexpr int kTileB = tile_b_bytes<BN>();
  constexpr int kBN = BN;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;
  uint8_t* sB = smem + kStages * kTileA;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * (kTileA + kTileB));
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + kStages);
  volatile int* s_ok = reinterpret_cast<volatile int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  const bool split = g.k_chunk > 0;
  const int kbase = split ? blockIdx.z * g.k_chunk : 0;
  const int klen = split ? min(g.k_chunk, g.K - kbase) : g.K;
  const int T = klen / kBK;
  float* Cout = (split && g.C) ? g.C + (size_t)blockIdx.z * g.M * g.ldc : g.C;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(tmem_cols<BN>()));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *s_ok = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  auto load_tile = [&](int t, int s) {
    const int k0 = kbase + t * kBK;
    const uint32_t a0 = smem_u32(sA + s * kTileA), b0 = smem_u32(sB + s * kTileB);
    // 128 rows x 8 chunks of 16 bytes for A, BN x 8 for B
    for (int c = tid; c < kBM * 8; c += kGemmThreads) {
      const int r = c >> 3, j = c & 7;
      const int row = min(m0 + r, g.M - 1);
      cp_async16(a0 + core_off(r, j * 8), g.A + (size_t)row * g.K + k0 + j * 8);
    }
    for (int c = tid; c < kBN * 8; c += kGemmThreads) {
      const int r = c >> 3, j = c & 7;
      const int row = min(n0 + r, g.N - 1);
      cp_async16(b0 + core_off(r, j * 8), g.B + (size_t)row * g.K + k0 + j * 8);
    }
    cp_async_commit();
  };

  const uint32_t idesc = instr_desc(kBM, kBN);
  bool ok = true;
  int issued = 0;  // tiles whose MMAs were committed
  load_tile(0, 0);
  for (int t = 0; t < T; ++t) {
    const int s = t & 1;
    if (t + 1 < T) {
      const int s1 = (t + 1) & 1;
      // stage s1 last held tile t-1: thread 0 waits for its MMAs (bounded)
      // and tells the block, so every thread takes the same branch
      if (t >= 1) {
        if (tid == 0 && !mbar_wait(&bars[s1], ((t - 1) >> 1) & 1, g.spin_limit)) *s_ok = 0;
        __syncthreads();
        ok = *s_ok != 0;
        if (!ok) break;
      }
      load_tile(t + 1, s1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(sA + s * kTileA), b0 = smem_u32(sB + s * kTileB);
#pragma unroll
      for (int kk = 0; kk < kBK / 16; ++kk) {
        // two core matrices (16 elements) along K per MMA
        const uint64_t da = smem_desc(a0 + kk * 256, g.lbo, g.sbo);
        const uint64_t db = smem_desc(b0 + kk * 256, g.lbo, g.sbo);
        mma_bf16(tmem, da, db, idesc, (t > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(&bars[s]);
    }
    ++issued;
  }
  // wait for the last committed tile (its commit covers all earlier MMAs);
  // the host sizes split-K chunks so that every CTA has a K tile
  if (ok && issued > 0) {
    const int tl = issued - 1;
    if (tid == 0 && !mbar_wait(&bars[tl & 1], (tl >> 1) & 1, g.spin_limit)) *s_ok = 0;
  }
  __syncthreads();
  ok = *s_ok != 0;
  if (!ok) {
    // timed out: report it, then let this CTA's own work finish before the
    // tensor memory is freed -- its copies, and (thread 0, with the full
    // limit) the last committed MMAs, whose commit covers all earlier ones
    if (tid == 0) {
      atomicExch(g.err, 1);
      if (issued > 0) {
        const int tl = issued - 1;
        mbar_wait(&bars[tl & 1], (tl >> 1) & 1, kSpinLimit);
      }
    }
    cp_async_wait<0>();
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    const int row = m0 + warp * 32 + lane;
    // 16-byte stores where the rows allow them (4 floats of C, 8 BF16 of Cb)
    const bool vc = !Cout || ((g.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(Cout) & 15) == 0);
    const bool vb = !g.Cb || ((g.ldcb & 7) == 0 && (reinterpret_cast<uintptr_t>(g.Cb) & 15) == 0);
    for (int c0 = 0; c0 < kBN; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      store16(g, split, Cout, row, n0, c0, v, vc, vb);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(tmem_cols<BN>()));
}

}  // namespace tc
}  // namespace mst
