// Persistent BF16 tensor-core GEMM with TMA operand copies, for the
// network's large-M layers (M = cells, N <= 256, K <= 256):
//
//   C[M, N] (FP32) = A[M, K] (BF16, row-major) . B[N, K]^T (BF16, row-major)
//                    (+ bias[N]) (ReLU) (+ C) ; optional BF16 copy of C
//
// Each CTA keeps one 128-wide column block of B (all of K) resident in shared
// memory and walks its share of the 128-row tiles of A.  Warp 0 (one lane)
// copies tiles with cp.async.bulk.tensor through tensor maps of this GPU's
// own memory, in the 128-byte-swizzled K-major layout, into a ring of
// kTmaStages stages; warp 1 (one lane) issues tcgen05.mma (kind::f16, BF16 x
// BF16 -> FP32) into one of two tensor-memory accumulators and commits each
// stage back to the copier; warps 2-9 read the other accumulator with
// tcgen05.ld and store the tile (each warp 32 rows x 64 columns in two
// loads, released to the MMA thread once both are in registers; whole
// 32-byte sectors per store; the C values of a residual add loaded before the
// accumulator is waited for), so a tile's epilogue overlaps the next
// tile's copies and products.  Every wait is bounded (GemmArgs.spin_limit
// polls): on timeout a role flags the CTA and the error word, the others
// stop, the copier waits for its copies in flight and the MMA thread for its
// products (full limit), and the tensor memory is freed before the CTA ends.
#pragma once
#include <cuda.h>  // CUtensorMap (the type; maps are encoded through the runtime's driver entry point)

#include "tc_gemm.cuh"

namespace mst {
namespace tc {

constexpr int kTmaStages = 6;                // A ring
constexpr int kTmaEpiWarps = 8;              // 4 row quarters x 2 column halves
constexpr int kTmaThreads = 64 + 32 * kTmaEpiWarps;  // copier, MMA, epilogue
constexpr int kTmaTile = kBM * kBK * 2;      // one 128-row x 64-K BF16 tile: 16 KB
constexpr int kTmaMaxKT = 4;                 // K <= 256
// dynamic shared memory: B (kt tiles) + the A ring + barriers, from a
// 1024-byte-aligned base (the 128-byte swizzle repeats every 1024 bytes; the
// kernel checks the base and reports a misaligned one instead of copying);
// at least 80 KB so that at most two CTAs share an SM (two double
// accumulators of 128 columns fill its 512 TMEM columns).  The epilogue's
// registers (the C values of the residual add held across the wait) keep
// it to one CTA per SM in practice; the launch asks the occupancy.
__host__ __device__ constexpr int tma_smem_bytes(int kt) {
  return ((kt + kTmaStages) * kTmaTile + 256) < 80 * 1024 ? 80 * 1024
                                                          : (kt + kTmaStages) * kTmaTile + 256;
}

// bounded wait that also gives up once another role has flagged the CTA
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* bar, uint32_t parity, unsigned limit,
                                                   volatile int* abort) {
  for (unsigned i = 0; i < limit; i += 256) {
    if (*abort) return false;
    if (mbar_wait(bar, parity, limit - i < 256 ? limit - i : 256)) return true;
  }
  return false;
}

// shared-memory matrix descriptor of a 128-byte-swizzled K-major tile
// (rows of 128 bytes, 8-row groups 1024 bytes apart)
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused when swizzled)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;             // descriptor version of this architecture
  d |= (uint64_t)2 << 61;             // layout: 128-byte swizzle
  return d;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// 2D tiled copy global -> shared, completing on bar's transaction count
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
      "{%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// 32 accumulator columns of this warp's 32 TMEM lanes (one per thread), the
// load and its completion wait in one statement so that no use of the
// registers can be scheduled before the wait
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 32-byte (one sector) global load / store of 8 floats; the address is
// 32-byte aligned
__device__ __forceinline__ void ld8(const float* p, float x[8]) {
  asm volatile("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=f"(x[0]), "=f"(x[1]), "=f"(x[2]), "=f"(x[3]), "=f"(x[4]), "=f"(x[5]),
                 "=f"(x[6]), "=f"(x[7])
               : "l"(p));
}
__device__ __forceinline__ void st8(float* p, const float x[8]) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(x[0]),
               "f"(x[1]), "f"(x[2]), "f"(x[3]), "f"(x[4]), "f"(x[5]), "f"(x[6]), "f"(x[7])
               : "memory");
}

struct TmaGemm {
  GemmArgs g;
  int kt;        // K / 64
  int n_ntiles;  // 128-wide column blocks of N
  int m_tiles;   // 128-row tiles of M
};

__global__ void __launch_bounds__(kTmaThreads, 1)
    k_gemm_tma(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
               const TmaGemm t) {
  constexpr int S = kTmaStages;
  extern __shared__ __align__(1024) uint8_t smem[];
  const GemmArgs& g = t.g;
  uint8_t* sB = smem;
  uint8_t* sA = smem + t.kt * kTmaTile;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sA + S * kTmaTile);
  uint64_t* full = bars;             // [S] a stage's copy landed
  uint64_t* empty = bars + S;        // [S] a stage's products are done
  uint64_t* bfull = bars + 2 * S;    // B landed
  uint64_t* accf = bars + 2 * S + 1; // [2] an accumulator holds a finished tile
  uint64_t* acce = bars + 2 * S + 3; // [2] an accumulator was read out
  uint64_t* drain = bars + 2 * S + 5;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * S + 6);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n0 = (blockIdx.x % t.n_ntiles) * kBN;
  const int m_first = blockIdx.x / t.n_ntiles, m_step = gridDim.x / t.n_ntiles;
  const unsigned lim = g.spin_limit;

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(2 * kBN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(bfull, 1);
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], kTmaEpiWarps);
    }
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // the swizzled layout needs a 1024-byte-aligned base: otherwise report
    // it and copy nothing
    *abort = (smem_u32(smem) & 1023) ? 1 : 0;
    if (*abort) atomicExch(g.err, 2);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {
      // copier: B once, then the A tiles of this CTA's rows through the ring
      bool ok = !*abort;
      uint32_t last_ph[S];
      bool used[S];
      for (int s = 0; s < S; ++s) used[s] = false;
      if (ok) {
        mbar_expect_tx(bfull, (uint32_t)(t.kt * kTmaTile));
        for (int k = 0; k < t.kt; ++k)
          tma_load_2d(smem_u32(sB + k * kTmaTile), &mapB, k * kBK, n0, bfull);
      }
      const bool b_issued = ok;
      int s = 0;
      uint32_t ph = 0;
      for (int m = m_first; m < t.m_tiles && ok; m += m_step) {
        for (int k = 0; k < t.kt; ++k) {
          if (!mbar_wait_or_abort(&empty[s], ph ^ 1, lim, abort)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&full[s], (uint32_t)kTmaTile);
          tma_load_2d(smem_u32(sA + s * kTmaTile), &mapA, k * kBK, m * kBM, &full[s]);
          used[s] = true;
          last_ph[s] = ph;
          if (++s == S) {
            s = 0;
            ph ^= 1;
          }
        }
      }
      if (!ok) {
        *abort = 1;
        atomicCAS(g.err, 0, 1);
      }
      // every copy of this CTA has landed before it ends
      if (b_issued) mbar_wait(bfull, 0, kSpinLimit);
      for (int q = 0; q < S; ++q)
        if (used[q]) mbar_wait(&full[q], last_ph[q], kSpinLimit);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      const uint32_t idesc = instr_desc(kBM, kBN);
      bool ok = mbar_wait_or_abort(bfull, 0, lim, abort);
      int s = 0, i = 0;
      uint32_t ph = 0;
      bool any = false;
      for (int m = m_first; m < t.m_tiles && ok; m += m_step, ++i) {
        const int b = i & 1;
        const uint32_t aph = (uint32_t)(i >> 1) & 1;
        if (!mbar_wait_or_abort(&acce[b], aph ^ 1, lim, abort)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t acc = tmem + (uint32_t)(b * kBN);
        for (int k = 0; k < t.kt; ++k) {
          if (!mbar_wait_or_abort(&full[s], ph, lim, abort)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t a0 = smem_u32(sA + s * kTmaTile), b0 = smem_u32(sB + k * kTmaTile);
#pragma unroll
          for (int kk = 0; kk < kBK / 16; ++kk)
            // K = 16 per product: 32 bytes further along the swizzled rows
            mma_bf16(acc, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), idesc,
                     (k > 0 || kk > 0) ? 1u : 0u);
          any = true;
          mma_commit(&empty[s]);
          if (++s == S) {
            s = 0;
            ph ^= 1;
          }
        }
        if (!ok) break;
        mma_commit(&accf[b]);
      }
      if (!ok) {
        *abort = 1;
        atomicCAS(g.err, 0, 1);
      }
      // every product of this CTA is done before the tensor memory is freed
      if (any) {
        mma_commit(drain);
        mbar_wait(drain, 0, kSpinLimit);
      }
    }
  } else {
    // epilogue warps 2-9: warp w reads TMEM lanes 32 (w % 4).. (its rows),
    // columns [64 h, 64 h + 64) with h = (w - 2) / 4
    const int q = warp & 3, h = (warp - 2) >> 2;
    const int cb = h * (kBN / 2);
    const bool vc = !g.C || ((g.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(g.C) & 15) == 0);
    const bool vb = !g.Cb || ((g.ldcb & 7) == 0 && (reinterpret_cast<uintptr_t>(g.Cb) & 15) == 0);
    // whole sectors: C rows 32-byte aligned
    const bool v32 = !g.C || ((g.ldc & 7) == 0 && (reinterpret_cast<uintptr_t>(g.C) & 31) == 0);
    int i = 0;
    for (int m = m_first; m < t.m_tiles; m += m_step, ++i) {
      const int b = i & 1;
      const uint32_t aph = (uint32_t)(i >> 1) & 1;
      const int row = m * kBM + q * 32 + lane;
      // warp-uniform (the TMEM loads below are .sync.aligned): every row of
      // the warp inside M, all 64 columns inside N, aligned rows
      const bool fast =
          __all_sync(0xffffffffu, row < g.M && n0 + cb + kBN / 2 <= g.N && v32 && vb) != 0;
      // the residual add's C values do not depend on the products: their
      // loads are in flight while the accumulator is still being formed
      const bool pre = fast && g.accumulate_c && g.C;
      float prev[kBN / 2];
      if (pre) {
        const float* p = g.C + (size_t)row * g.ldc + n0 + cb;
#pragma unroll
        for (int j = 0; j < kBN / 16; ++j) ld8(p + 8 * j, &prev[8 * j]);
      }
      int go = 0;
      if (lane == 0) go = mbar_wait_or_abort(&accf[b], aph, lim, abort) ? 1 : 0;
      go = __shfl_sync(0xffffffffu, go, 0);
      if (!go) {
        if (lane == 0) {
          *abort = 1;
          atomicCAS(g.err, 0, 1);
        }
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acc = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kBN + cb);
      if (fast) {
        const int col0 = n0 + cb;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          float v[32];
          tmem_ld32(acc + 32 * half, v);
          if (half == 1) {
            // the accumulator is in registers: the MMA thread may reuse it
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[b]);
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int c = 32 * half + 8 * j;  // column within the warp's 64
            float x[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              float y = v[8 * j + k];
              if (g.bias) y += __ldg(g.bias + col0 + c + k);
              if (g.relu) y = fmaxf(y, 0.f);
              x[k] = y;
            }
            if (g.C) {
              float o[8];
#pragma unroll
              for (int k = 0; k < 8; ++k) o[k] = pre ? x[k] + prev[c + k] : x[k];
              st8(g.C + (size_t)row * g.ldc + col0 + c, o);
            }
            if (g.Cb) {
              uint32_t w[4];
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                const __nv_bfloat162 b2 = __floats2bfloat162_rn(x[2 * k], x[2 * k + 1]);
                w[k] = *reinterpret_cast<const uint32_t*>(&b2);
              }
              *reinterpret_cast<uint4*>(g.Cb + (size_t)row * g.ldcb + col0 + c) =
                  make_uint4(w[0], w[1], w[2], w[3]);
            }
          }
        }
      } else {
        // ragged columns, rows past M or unaligned rows: 16 at a time
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          float v[32];
          tmem_ld32(acc + 32 * half, v);
          store16(g, false, g.C, row, n0, cb + 32 * half, &v[0], vc, vb);
          store16(g, false, g.C, row, n0, cb + 32 * half + 16, &v[16], vc, vb);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&acce[b]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * kBN));
}

// Split-K variant for the weight gradients (M, N <= 256, K = the cells):
// CTA (m, n, z) forms the 128x128 partial product of its K chunk and stores
// it to C + z * M * ldc (no bias / ReLU; the caller adds the chunks in
// order).  Warp 0 copies A and B tiles (128 x 64 each) with
// cp.async.bulk.tensor into a ring of kSplitStages stages, warp 1 issues
// the products into one TMEM accumulator, warps 2-5 store it.  Two CTAs per
// SM.  The same bounded waits and drain as k_gemm_tma.
constexpr int kSplitStages = 3;
constexpr int kSplitThreads = 192;
__host__ __device__ constexpr int split_smem_bytes() { return kSplitStages * 2 * kTmaTile + 256; }

__global__ void __launch_bounds__(kSplitThreads)
    k_gemm_tma_split(const __grid_constant__ CUtensorMap mapA,
                     const __grid_constant__ CUtensorMap mapB, const GemmArgs g) {
  constexpr int S = kSplitStages;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA = smem;
  uint8_t* sB = smem + S * kTmaTile;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + S * kTmaTile);
  uint64_t* full = bars;           // [S] a stage's A and B landed
  uint64_t* empty = bars + S;      // [S] a stage's products are done
  uint64_t* accf = bars + 2 * S;   // the accumulator holds the chunk's product
  uint64_t* drain = bars + 2 * S + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * S + 2);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  const int kbase = blockIdx.z * g.k_chunk;
  const int T = min(g.k_chunk, g.K - kbase) / kBK;
  float* Cout = g.C + (size_t)blockIdx.z * g.M * g.ldc;
  const unsigned lim = g.spin_limit;

  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(kBN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    for (int q = 0; q < S; ++q) {
      mbar_init(&full[q], 1);
      mbar_init(&empty[q], 1);
    }
    mbar_init(accf, 1);
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort = ((smem_u32(smem) & 1023) || T < 1) ? 1 : 0;
    if (*abort) atomicExch(g.err, 2);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {
      bool ok = !*abort;
      uint32_t last_ph[S];
      bool used[S];
      for (int q = 0; q < S; ++q) used[q] = false;
      int st = 0;
      uint32_t ph = 0;
      for (int k = 0; k < T && ok; ++k) {
        if (!mbar_wait_or_abort(&empty[st], ph ^ 1, lim, abort)) {
          ok = false;
          break;
        }
        mbar_expect_tx(&full[st], (uint32_t)(2 * kTmaTile));
        tma_load_2d(smem_u32(sA + st * kTmaTile), &mapA, kbase + k * kBK, m0, &full[st]);
        tma_load_2d(smem_u32(sB + st * kTmaTile), &mapB, kbase + k * kBK, n0, &full[st]);
        used[st] = true;
        last_ph[st] = ph;
        if (++st == S) {
          st = 0;
          ph ^= 1;
        }
      }
      if (!ok) {
        *abort = 1;
        atomicCAS(g.err, 0, 1);
      }
      for (int q = 0; q < S; ++q)
        if (used[q]) mbar_wait(&full[q], last_ph[q], kSpinLimit);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = instr_desc(kBM, kBN);
      bool ok = !*abort, any = false;
      int st = 0;
      uint32_t ph = 0;
      for (int k = 0; k < T && ok; ++k) {
        if (!mbar_wait_or_abort(&full[st], ph, lim, abort)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a0 = smem_u32(sA + st * kTmaTile), b0 = smem_u32(sB + st * kTmaTile);
#pragma unroll
        for (int kk = 0; kk < kBK / 16; ++kk)
          mma_bf16(tmem, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), idesc,
                   (k > 0 || kk > 0) ? 1u : 0u);
        any = true;
        mma_commit(&empty[st]);
        if (++st == S) {
          st = 0;
          ph ^= 1;
        }
      }
      if (ok) {
        mma_commit(accf);
      } else {
        *abort = 1;
        atomicCAS(g.err, 0, 1);
      }
      if (any) {
        mma_commit(drain);
        mbar_wait(drain, 0, kSpinLimit);
      }
    }
  } else {
    // epilogue warps 2-5: warp w reads TMEM lanes 32 (w % 4).. = its rows
    const int q = warp & 3;
    int go = 0;
    if (lane == 0) go = mbar_wait_or_abort(accf, 0, lim, abort) ? 1 : 0;
    go = __shfl_sync(0xffffffffu, go, 0);
    if (!go) {
      if (lane == 0) {
        *abort = 1;
        atomicCAS(g.err, 0, 1);
      }
    } else {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const bool vc = (g.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(Cout) & 15) == 0;
      const int row = m0 + q * 32 + lane;
      for (int c0 = 0; c0 < kBN; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        store16(g, true, Cout, row, n0, c0, v, vc, true);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBN));
}

}  // namespace tc
}  // namespace mst
