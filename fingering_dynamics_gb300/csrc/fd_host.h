// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>

#include "../../include/fdlbm.h"

namespace fd {

// Message of the last failing call on this host thread (fd_last_error).
void set_error(const char* fmt, ...);

#define FD_REQUIRE(cond, code, ...)  \
  do {                               \
    if (!(cond)) {                   \
      ::fd::set_error(__VA_ARGS__);  \
      return (code);                 \
    }                                \
  } while (0)

inline int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return FD_ERR_CUDA;
  }
  return FD_OK;
}

inline int check_params(const fd_params* p) {
  FD_REQUIRE(p != nullptr, FD_ERR_ARG, "params is NULL");
  FD_REQUIRE(p->H >= 2 && p->W >= 2, FD_ERR_SHAPE, "lattice %dx%d too small", p->H, p->W);
  FD_REQUIRE(p->variant == FD_VARIANT_PERIODIC || p->variant == FD_VARIANT_WALLS ||
                 p->variant == FD_VARIANT_PERIODIC_XY,
             FD_ERR_ARG, "unknown variant %d", p->variant);
  FD_REQUIRE(p->variant != FD_VARIANT_WALLS || p->H >= 3, FD_ERR_SHAPE,
             "the walled variant needs H >= 3 (walls act on rows 1 and H-2)");
  return FD_OK;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Raise a kernel's dynamic shared-memory limit to `bytes` once per device
// (the attribute is per device; `done` is the caller's per-kernel bit set of
// devices already configured, safe to share between host threads).
template <typename K>
inline cudaError_t ensure_smem_attr(K kernel, int bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

}  // namespace fd
