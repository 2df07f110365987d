// Library-level C ABI: version, error reporting and the fused-step dispatch.
#include <cstdio>
#include <cstring>

#include "fd_host.h"

namespace fd {

namespace {
thread_local char g_last_error[512] = "";
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int fused_f64(const fd_params& p, const uint16_t* mask, const double* inlet_ux, void* pa, void* pb, void* sa, void* sb,
              int nsteps, int R, cudaStream_t st);
int fused_f32(const fd_params& p, const uint16_t* mask, const double* inlet_ux, void* pa, void* pb, void* sa, void* sb,
              int nsteps, int R, cudaStream_t st);

// Rows one warp marches: enough warps to fill the GPU several times over,
// few enough that the two halo rows of g per strip stay a small overhead.
int auto_rows(int H, int W, int vec) {
  const long long chunks = ((long long)(W / vec) + 29) / 30;
  long long R = (long long)H * chunks / (152LL * 24);
  if (R < 4) R = 4;
  if (R > 64) R = 64;
  if (R > H) R = H;
  return (int)R;
}

}  // namespace fd

using namespace fd;

extern "C" {

int fd_abi_version(void) { return FDLBM_ABI_VERSION; }

const char* fd_last_error(void) { return g_last_error; }

int fd_fused_step(const fd_params* prm, int dtype, const uint16_t* mask, const double* inlet_ux, void* pop_a,
                  void* pop_b, void* side_a, void* side_b, int nsteps, int rows_per_warp, void* stream) {
  if (int r = check_params(prm)) return r;
  FD_REQUIRE(dtype == FD_F64 || dtype == FD_F32, FD_ERR_DTYPE, "fd_fused_step: dtype %d not supported", dtype);
  FD_REQUIRE(mask && inlet_ux && pop_a && pop_b && side_a && side_b, FD_ERR_ARG, "fd_fused_step: NULL pointer");
  FD_REQUIRE(pop_a != pop_b && side_a != side_b, FD_ERR_ARG, "fd_fused_step: ping-pong buffers must differ");
  FD_REQUIRE(nsteps >= 0, FD_ERR_ARG, "fd_fused_step: negative step count");
#ifndef FD_F32_VEC
#define FD_F32_VEC 4
#endif
  const int vec = dtype == FD_F64 ? 2 : FD_F32_VEC;
  FD_REQUIRE(prm->W % vec == 0 && prm->W >= 2 * vec && prm->H >= 3, FD_ERR_SHAPE,
             "fd_fused_step: W must be a multiple of %d and >= %d, H >= 3 (got %dx%d)", vec, 2 * vec, prm->H, prm->W);
  FD_REQUIRE(((uintptr_t)pop_a | (uintptr_t)pop_b | (uintptr_t)mask) % 16 == 0, FD_ERR_ARG,
             "fd_fused_step: buffers must be 16-byte aligned");
  const int R = rows_per_warp > 0 ? rows_per_warp : auto_rows(prm->H, prm->W, vec);
  if (nsteps == 0) return FD_OK;
  const int r = dtype == FD_F64
                    ? fused_f64(*prm, mask, inlet_ux, pop_a, pop_b, side_a, side_b, nsteps, R, as_stream(stream))
                    : fused_f32(*prm, mask, inlet_ux, pop_a, pop_b, side_a, side_b, nsteps, R, as_stream(stream));
  if (r != FD_OK) return check_launch("fd_fused_step");
  return FD_OK;
}

}  // extern "C"
