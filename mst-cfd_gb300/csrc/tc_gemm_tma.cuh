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
// stage back to the copier; warps 2-5 read the other accumulator with
// tcgen05.ld and store the tile, so a tile's epilogue overlaps the next
// tile's copies and products.  Every wait is bounded (GemmArgs.spin_limit
// polls): on timeout a role flags the CTA and the error word, the others
// stop, the copier waits for its copies in flight and the MMA thread for its
// products (full limit), and the tensor memory is freed before the CTA ends.
#pragma once
#include <cuda.h>  // CUtensorMap (the type; maps are encoded through the runtime's driver entry point)

#include "tc_gemm.cuh"

namespace mst {
namespace tc {

constexpr int kTmaStages = 3;                // A ring
constexpr int kTmaThreads = 192;             // copier, MMA, 4 epilogue warps
constexpr int kTmaTile = kBM * kBK * 2;      // one 128-row x 64-K BF16 tile: 16 KB
constexpr int kTmaMaxKT = 4;                 // K <= 256
// dynamic shared memory: B (kt tiles) + the A ring + barriers, from a
// 1024-byte-aligned base (the 128-byte swizzle repeats every 1024 bytes; the
// kernel checks the base and reports a misaligned one instead of copying);
// at least 80 KB so that at most two CTAs share an SM (two double
// accumulators of 128 columns fill its 512 TMEM columns), at most 112.25 KB
// so that two do
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

struct TmaGemm {
  GemmArgs g;
  int kt;        // K / 64
  int n_ntiles;  // 128-wide column blocks of N
  int m_tiles;   // 128-row tiles of M
};

__global__ void __launch_bounds__(kTmaThreads)
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
      mbar_init(&acce[b], 4);
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
    // epilogue warps 2-5: warp w reads TMEM lanes 32 (w % 4).. = its rows
    const int q = warp & 3;
    const bool vc = !g.C || ((g.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(g.C) & 15) == 0);
    const bool vb = !g.Cb || ((g.ldcb & 7) == 0 && (reinterpret_cast<uintptr_t>(g.Cb) & 15) == 0);
    int i = 0;
    for (int m = m_first; m < t.m_tiles; m += m_step, ++i) {
      const int b = i & 1;
      const uint32_t aph = (uint32_t)(i >> 1) & 1;
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
      const int row = m * kBM + q * 32 + lane;
      for (int c0 = 0; c0 < kBN; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * kBN + c0), v);
        store16(g, false, g.C, row, n0, c0, v, vc, vb);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[b]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(2 * kBN));
}

}  // namespace tc
}  // namespace mst
