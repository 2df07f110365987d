// Instantiations of the shared-memory-staged fused step (fd_fused_tma.cuh)
// and the device status word.
#include "fd_fused_tma.cuh"
#include "fd_host.h"

namespace fd {

template <typename SF, bool STOCH>
int fused_tma_r(const fd_params& p, const fd_storage& st, const DevCoef& c, const uint16_t* mask,
                const double* inlet_ux, void* pa, void* pb, void* sa, void* sb, int nsteps, int R, cudaStream_t s) {
  const bool scaled = st.f_scale_log2 != 0 || st.g_scale_log2 != 0;
  if (scaled)
    return launch_fused_tma<SF, FD_TMA_NT, tma_ring_depth<SF>(), true, STOCH>(p, c, mask, inlet_ux, (char*)pa, (char*)pb,
                                                                   (float*)sa, (float*)sb, nsteps, R, st.seed, s);
  return launch_fused_tma<SF, FD_TMA_NT, tma_ring_depth<SF>(), false, STOCH>(p, c, mask, inlet_ux, (char*)pa, (char*)pb,
                                                                  (float*)sa, (float*)sb, nsteps, R, st.seed, s);
}

template <typename SF>
int fused_tma_t(const fd_params& p, const fd_storage& st, const DevCoef& c, const uint16_t* mask,
                const double* inlet_ux, void* pa, void* pb, void* sa, void* sb, int nsteps, int R, cudaStream_t s) {
  if (st.rounding == FD_ROUND_STOCHASTIC)
    return fused_tma_r<SF, true>(p, st, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R, s);
  return fused_tma_r<SF, false>(p, st, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R, s);
}

int fused_tma(const fd_params& p, const fd_storage& st, const DevCoef& c, const uint16_t* mask,
              const double* inlet_ux, void* pa, void* pb, void* sa, void* sb, int nsteps, int R, cudaStream_t s) {
  switch (st.dtype) {
    case FD_F16: return fused_tma_t<__half>(p, st, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R, s);
    case FD_BF16: return fused_tma_t<__nv_bfloat16>(p, st, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R, s);
    default:
      return launch_fused_tma<float, FD_TMA_NT, tma_ring_depth<float>(), false, false>(p, c, mask, inlet_ux, (char*)pa, (char*)pb,
                                                                         (float*)sa, (float*)sb, nsteps, R, 0, s);
  }
}

int tma_band_width() { return FD_TMA_NT; }

template <typename SF, bool SCALED, bool STOCH>
int tma_strips_t(const fd_params& p, const DevCoef& c, const uint16_t* mask, const double* inlet_ux, const void* src,
                 void* dst, const void* side_in, void* side_out, int R, int strip0, int nstrips, uint32_t seed,
                 cudaStream_t s) {
  constexpr int NS = tma_ring_depth<SF>();
  DevArgs<SF> a = tma_args<SF, FD_TMA_NT, NS, SCALED, STOCH>(p, c, mask, inlet_ux, R);
  tma_set_step(a, (const char*)src, (char*)dst, (float*)side_in, (float*)side_out, seed);
  TmaMaps tm;
  if (int r = tma_maps<SF, FD_TMA_NT>(a, (const char*)src, tm)) return r;
  return launch_tma_strips<SF, FD_TMA_NT, NS, SCALED, STOCH>(a, tm, strip0, nstrips, s);
}

template <typename SF>
int tma_strips_r(const fd_params& p, const fd_storage& st, const DevCoef& c, const uint16_t* mask,
                 const double* inlet_ux, const void* src, void* dst, const void* side_in, void* side_out, int R,
                 int strip0, int nstrips, uint32_t seed, cudaStream_t s) {
  const bool scaled = st.f_scale_log2 != 0 || st.g_scale_log2 != 0;
  const bool sr = st.rounding == FD_ROUND_STOCHASTIC;
  if (scaled)
    return sr ? tma_strips_t<SF, true, true>(p, c, mask, inlet_ux, src, dst, side_in, side_out, R, strip0, nstrips, seed, s)
              : tma_strips_t<SF, true, false>(p, c, mask, inlet_ux, src, dst, side_in, side_out, R, strip0, nstrips, seed, s);
  return sr ? tma_strips_t<SF, false, true>(p, c, mask, inlet_ux, src, dst, side_in, side_out, R, strip0, nstrips, seed, s)
            : tma_strips_t<SF, false, false>(p, c, mask, inlet_ux, src, dst, side_in, side_out, R, strip0, nstrips, seed, s);
}

// One step of the staged kernel over strips strip0 .. strip0 + nstrips - 1 of
// R rows each (R > 0); `seed` is the step's seed (the call's seed plus the
// step index), as in fused_tma.
int fused_tma_strips(const fd_params& p, const fd_storage& st, const DevCoef& c, const uint16_t* mask,
                     const double* inlet_ux, const void* src, void* dst, const void* side_in, void* side_out, int R,
                     int strip0, int nstrips, uint32_t seed, cudaStream_t s) {
  switch (st.dtype) {
    case FD_F16:
      return tma_strips_r<__half>(p, st, c, mask, inlet_ux, src, dst, side_in, side_out, R, strip0, nstrips, seed, s);
    case FD_BF16:
      return tma_strips_r<__nv_bfloat16>(p, st, c, mask, inlet_ux, src, dst, side_in, side_out, R, strip0, nstrips,
                                         seed, s);
    default:
      return tma_strips_t<float, false, false>(p, c, mask, inlet_ux, src, dst, side_in, side_out, R, strip0, nstrips,
                                               seed, s);
  }
}

int batch_device_error(unsigned* out, bool clear);
int dev_device_error(unsigned* out, bool clear);
int batch_selftest_wait_timeout(unsigned polls, cudaStream_t s);

// One thread waits, through the staged kernel's bounded wait, on an mbarrier
// that nothing arrives on: the wait gives up after `polls` polls and latches
// bit 0 of the device error word (the failure path of the kernel, exercised
// without a fault or a hang).
__global__ void k_selftest_wait_timeout(unsigned polls) {
  __shared__ uint64_t bar;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  mbar_wait(&bar, 0u, polls);
}

}  // namespace fd

extern "C" int fd_selftest_wait_timeout(unsigned polls, int unit, void* stream) {
  FD_REQUIRE(polls >= 1 && polls <= (1u << 20), FD_ERR_ARG, "fd_selftest_wait_timeout: polls in [1, 2^20]");
  FD_REQUIRE(unit == 0 || unit == 1, FD_ERR_ARG, "fd_selftest_wait_timeout: unit 0 (single lattice) or 1 (batch)");
  if (unit == 1) {
    fd::batch_selftest_wait_timeout(polls, fd::as_stream(stream));
  } else {
    fd::k_selftest_wait_timeout<<<1, 1, 0, fd::as_stream(stream)>>>(polls);
  }
  return fd::check_launch("fd_selftest_wait_timeout");
}

extern "C" int fd_device_status(unsigned* out, int clear) {
  FD_REQUIRE(out != nullptr, FD_ERR_ARG, "fd_device_status: NULL pointer");
  unsigned single = 0, batch = 0, reg = 0;
  if (fd::device_error_word(&single, clear != 0) != FD_OK || fd::batch_device_error(&batch, clear != 0) != FD_OK ||
      fd::dev_device_error(&reg, clear != 0) != FD_OK)
    return fd::check_launch("fd_device_status");
  *out = single | batch | reg;
  return FD_OK;
}
