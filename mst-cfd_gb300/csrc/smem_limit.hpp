// Per-device record of a kernel's raised dynamic shared-memory limit.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

namespace mst {

// Raises a kernel's dynamic shared-memory limit on the current device the
// first time that device launches it.  The attribute belongs to the
// (kernel, device) pair, so `done` records one bit per device index; two
// threads racing on a first launch both set it, which is harmless.
template <class K>
cudaError_t ensure_smem_limit(K* kernel, int bytes, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  done.fetch_or(bit, std::memory_order_acq_rel);
  return cudaSuccess;
}

}  // namespace mst
