// A fused-step entry point that allocates nothing.
//
// fd_fused_step_packed needs two caller buffers for the Zou-He boundary
// values (psi_x, psi_y, mu at columns 0 and W-1) because every iteration
// reads the previous iteration's values and writes new ones.  Some callers
// cannot provide the second one: a host whose memory manager owns all of
// device memory (a framework's caching allocator, or an arena reserved at
// start-up) and does not let a library call cudaMalloc behind its back, or a
// host that allocates everything once before it starts stepping.  For them,
// fd_fused_step_packed_noalloc keeps the second boundary buffer in a fixed
// array in device memory that belongs to this library, so the caller passes
// only its own state buffers.
#include <cuda.h>

#include <mutex>

#include "fd_host.h"

namespace fd {

// The library's fixed boundary buffer (see fd_fused_step_packed_noalloc).
static __device__ __align__(256) float g_noalloc_side[6 * 16384];

namespace {

// Largest lattice height the fixed boundary buffer covers: 6 * 16384 floats
// = 384 KiB, reserved on every GPU that loads this library until the process
// exits.
constexpr int kNoAllocMaxH = 16384;
static_assert(sizeof(g_noalloc_side) == sizeof(float) * 6 * kNoAllocMaxH, "buffer size");
constexpr int kMaxDevices = 64;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

// cuCtxGetCurrent from the driver through the runtime's entry-point query (the
// library does not link libcuda); null if the driver does not offer it.
CtxGetCurrentFn ctx_get_current_fn() {
  static const CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (CtxGetCurrentFn) nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

std::mutex g_setup_mutex;
struct SideScratch {
  CUcontext ctx;
  float* ptr;
};
SideScratch g_side[kMaxDevices] = {};

// Device address of g_noalloc_side on the current device.  The host-side name
// is only a stand-in for the symbol, so the address is looked up with
// cudaGetSymbolAddress, once per device and context: a context torn down and
// created again (cudaDeviceReset) is looked up afresh.
int side_scratch(float** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("fd_fused_step_packed_noalloc");
  FD_REQUIRE(dev >= 0 && dev < kMaxDevices, FD_ERR_ARG, "fd_fused_step_packed_noalloc: device %d out of range", dev);
  const CtxGetCurrentFn get_ctx = ctx_get_current_fn();
  FD_REQUIRE(get_ctx != nullptr, FD_ERR_CUDA, "fd_fused_step_packed_noalloc: cuCtxGetCurrent is not available");
  CUcontext ctx = nullptr;  // null until the runtime has made the device's context current on this thread
  if (get_ctx(&ctx) != CUDA_SUCCESS) ctx = nullptr;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (ctx == nullptr || g_side[dev].ptr == nullptr || g_side[dev].ctx != ctx) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_side);
    if (e != cudaSuccess) {
      set_error("fd_fused_step_packed_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return FD_ERR_CUDA;
    }
    FD_REQUIRE(get_ctx(&ctx) == CUDA_SUCCESS && ctx != nullptr, FD_ERR_CUDA,
               "fd_fused_step_packed_noalloc: no current CUDA context");
    g_side[dev] = SideScratch{ctx, static_cast<float*>(p)};
  }
  *out = g_side[dev].ptr;
  return FD_OK;
}

}  // namespace
}  // namespace fd

extern "C" int fd_fused_step_packed_noalloc(const fd_params* prm, const fd_storage* st, const uint16_t* mask,
                                            const double* inlet_ux, void* pop_a, void* pop_b, void* side,
                                            int nsteps, int rows_per_warp, void* stream) {
  if (int r = fd::check_params(prm)) return r;
  FD_REQUIRE(prm->H <= fd::kNoAllocMaxH, FD_ERR_SCRATCH,
             "fd_fused_step_packed_noalloc: H = %d exceeds the fixed boundary buffer (H <= %d); "
             "use fd_fused_step_packed with caller buffers",
             prm->H, fd::kNoAllocMaxH);
  FD_REQUIRE(side != nullptr, FD_ERR_ARG, "fd_fused_step_packed_noalloc: NULL pointer");
  float* scratch = nullptr;
  if (int r = fd::side_scratch(&scratch)) return r;
  // even iterations read the caller's buffer and write the fixed one, odd
  // iterations the reverse
  if (int r = fd_fused_step_packed(prm, st, mask, inlet_ux, pop_a, pop_b, side, scratch, nsteps, rows_per_warp,
                                   stream))
    return r;
  if (nsteps % 2) {
    // the newest boundary values are in the fixed buffer: hand them back
    const cudaError_t e = cudaMemcpyAsync(side, scratch, sizeof(float) * 6 * (size_t)prm->H,
                                          cudaMemcpyDeviceToDevice, fd::as_stream(stream));
    if (e != cudaSuccess) {
      fd::set_error("fd_fused_step_packed_noalloc: boundary copy failed: %s", cudaGetErrorString(e));
      return FD_ERR_CUDA;
    }
  }
  return FD_OK;
}
