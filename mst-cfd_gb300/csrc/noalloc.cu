// mst_solve_device_noalloc: one residual evaluation and explicit update on
// caller-owned device buffers, with no device allocation in the call.
//
// Who needs it: programs that embed the solver in a larger GPU application
// which owns every byte of device memory through its own pool or arena and
// does not allow raw cudaMalloc/cudaFree while it runs (cudaFree waits for
// the whole device, and a cudaMalloc can fail or fragment a pool that is
// already carved up), and time-critical loops that must not take those
// implicit device synchronisations.  Such a caller creates the context once
// at set-up (that call allocates the resident mesh), then calls this entry
// point as often as it likes with its own input and output buffers.
//
// Arithmetic: the context's precision; the state is the caller's FP64
// buffers, so on the FP32 path the update is done in FP64 (mst_solve keeps
// that path's state as float pairs) and the two agree to FP32 rounding.
//
// Scratch: the gradient and the per-tile norm partials that mst_solve keeps
// in context allocations live here in one file-scope device array of fixed
// size instead, so a mesh may have at most kMaxCells cells.  Every GPU that
// loads the library holds the array (about 8.1 MiB) until the process exits.
// All calls share it: two calls whose work overlaps on the GPU (from two
// host threads, or on two contexts of one device) race on it and must be
// serialised by the caller.  Each call writes every scratch word it reads
// before reading it, so nothing carries over from the previous call.
#include <cuda_runtime.h>

#include <string>

#include "ctx.hpp"

namespace {

constexpr int kMaxCells = 131072;
constexpr int kMaxTiles = (kMaxCells + mst::kTileCells - 1) / mst::kTileCells;
constexpr size_t kGradBytes = (size_t)kMaxCells * 8 * sizeof(double);
constexpr size_t kPartBytes = (size_t)kMaxTiles * mst::kNormSlots * sizeof(double);

static __device__ __align__(256) unsigned char g_scratch[kGradBytes + kPartBytes];

// Device address of g_scratch on the current device.  In host code the
// name g_scratch is only a stand-in, not a device address, so the address
// is looked up with cudaGetSymbolAddress with the device current.  The
// first call on a device is the set-up: it may load the library's device
// code onto that device, so it should come before any stream capture.
// The lookup is repeated on every call (it allocates nothing once the code
// is loaded), so an address never outlives a device reset.
mst_status scratch_for_current_device(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess || !p) {
    return mst_internal_fail(MST_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  }
  *out = p;
  return MST_OK;
}

bool overlaps(const void* a, const void* b, size_t n) {
  const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
  return x < y + n && y < x + n;
}

// linf[4] (max), l2[4] (sqrt of mean), mass (sum) from the per-tile partials;
// out[9] = dt of the call
__global__ void k_noalloc_norms(const double* __restrict__ part, int n_tiles,
                                int n_cells, double dt, double* __restrict__ out) {
  __shared__ double red[mst::kNormSlots][2];
  const int j = threadIdx.y;
  double x = 0.0;
  for (int i = threadIdx.x; i < n_tiles; i += blockDim.x) {
    const double v = part[(size_t)i * mst::kNormSlots + j];
    x = (j < 4) ? ((x < v) ? v : x) : x + v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, x, o);
    x = (j < 4) ? ((x < w) ? w : x) : x + w;
  }
  if ((threadIdx.x & 31) == 0) red[j][threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = red[j][0];
    const double w = red[j][1];
    acc = (j < 4) ? ((acc < w) ? w : acc) : acc + w;
    if (j >= 4 && j < 8) acc = sqrt(acc / (double)n_cells);
    out[j] = acc;
    if (j == 0) out[mst::kNormSlots] = dt;
  }
}

}  // namespace

extern "C" mst_status mst_solve_device_noalloc(mst_ctx* c, const double* q_dev,
                                               double* qnew_dev, double* r_dev,
                                               double* norms_dev) {
  if (!c || !q_dev || !qnew_dev) {
    return mst_internal_fail(MST_EINVAL, "NULL argument");
  }
  const int nC = c->dm.n_cells;
  if (nC > kMaxCells) {
    return mst_internal_fail(MST_EINVAL, "mst_solve_device_noalloc: mesh has " + std::to_string(nC) +
            " cells; the built-in scratch holds at most " + std::to_string(kMaxCells));
  }
  if (c->p.time_scheme != MST_TIME_EULER || c->p.dt_mode != MST_DT_FIXED) {
    return mst_internal_fail(MST_EUNSUPPORTED, "mst_solve_device_noalloc: the context must use "
                             "one Euler stage at a fixed dt (time_scheme MST_TIME_EULER, dt_mode "
                             "MST_DT_FIXED)");
  }
  const size_t bytes = (size_t)nC * 4 * sizeof(double);
  if (overlaps(q_dev, qnew_dev, bytes) || (r_dev && (overlaps(q_dev, r_dev, bytes) ||
                                                     overlaps(qnew_dev, r_dev, bytes)))) {
    return mst_internal_fail(MST_EINVAL, "mst_solve_device_noalloc: q_dev, qnew_dev and r_dev "
                             "must not overlap");
  }
  auto misaligned = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 31) != 0; };
  if (misaligned(q_dev) || misaligned(qnew_dev) || (r_dev && misaligned(r_dev))) {
    return mst_internal_fail(MST_EINVAL, "state buffers must be 32-byte aligned");
  }
  void* base = nullptr;
  mst_status st = scratch_for_current_device(&base);
  if (st != MST_OK) return st;
  void* grad = base;
  double* partials = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kGradBytes);

  const double4_32a* q = reinterpret_cast<const double4_32a*>(q_dev);
  const bool exact = c->p.precision == MST_PREC_FP64_EXACT;
  cudaError_t e = cudaSuccess;
  if (c->p.order == 2) {
    e = exact ? mst::exact::launch_gradient(c->p.precision, c->dm, q, grad,
                                            c->p.reference_quirks, c->stream)
              : mst::fast::launch_gradient(c->p.precision, c->dm, q, grad,
                                           c->p.reference_quirks, c->stream);
    if (e != cudaSuccess) {
      return mst_internal_fail(MST_ECUDA, std::string("gradient: ") + cudaGetErrorString(e));
    }
  }
  mst::StepArgs a{};
  a.q = q;
  a.qn = reinterpret_cast<double4_32a*>(qnew_dev);
  a.r_out = reinterpret_cast<double4_32a*>(r_dev);
  a.grad = grad;
  a.dt = c->p.dt;
  a.stage = 0;
  a.quirks = c->p.reference_quirks;
  a.limiter = c->p.limiter;
  mst::set_physics(a, c->p.inlet_q, c->p.viscous, c->p.mu, c->p.lambda, c->p.kappa,
                   c->p.cv);
  a.partials = norms_dev ? partials : nullptr;
  e = exact ? mst::exact::launch_flux_update(c->p.precision, c->p.flux, c->p.order, c->dm, a,
                                             0, c->stream)
            : mst::fast::launch_flux_update(c->p.precision, c->p.flux, c->p.order, c->dm, a,
                                            0, c->stream);
  if (e != cudaSuccess) {
    return mst_internal_fail(MST_ECUDA, std::string("flux_update: ") + cudaGetErrorString(e));
  }
  if (norms_dev) {
    k_noalloc_norms<<<1, dim3(64, mst::kNormSlots), 0, c->stream>>>(
        partials, c->dm.n_tiles, nC, c->p.dt, norms_dev);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      return mst_internal_fail(MST_ECUDA, std::string("norms: ") + cudaGetErrorString(e));
    }
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    return mst_internal_fail(MST_ECUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
  }
  return MST_OK;
}

