// Packed-storage fused step (deviation form, FP32 arithmetic) and the
// pack / unpack conversions, with their C ABI.
#include "fd_fused_dev.cuh"
#include "fd_host.h"

namespace fd {
// This unit's copy of the device status word (fd_fused_dev.cuh), which the
// register kernel latches; fd_device_status() combines it with the others.
int dev_device_error(unsigned* out, bool clear) { return device_error_word(out, clear); }
int fused_tma(const fd_params& p, const fd_storage& st, const DevCoef& c, const uint16_t* mask,
              const double* inlet_ux, void* pa, void* pb, void* sa, void* sb, int nsteps, int R, cudaStream_t s);
int tma_band_width();
namespace {

int check_storage(const fd_storage* s) {
  FD_REQUIRE(s != nullptr, FD_ERR_ARG, "storage descriptor is NULL");
  FD_REQUIRE(s->dtype == FD_F32 || s->dtype == FD_F16 || s->dtype == FD_BF16, FD_ERR_DTYPE,
             "packed storage supports FD_F32, FD_F16, FD_BF16 (got %d)", s->dtype);
  FD_REQUIRE(s->f_scale_log2 >= -30 && s->f_scale_log2 <= 30 && s->g_scale_log2 >= -30 && s->g_scale_log2 <= 30,
             FD_ERR_ARG, "storage scale exponents out of range");
  FD_REQUIRE(s->rounding == FD_ROUND_NEAREST || s->rounding == FD_ROUND_STOCHASTIC, FD_ERR_ARG,
             "storage rounding must be FD_ROUND_NEAREST or FD_ROUND_STOCHASTIC (got %d)", s->rounding);
  return FD_OK;
}

size_t packed_bytes(int H, int W, int dtype) {
  switch (dtype) {
    case FD_F16: return packed_layout<__half>(H, W).total;
    case FD_BF16: return packed_layout<__nv_bfloat16>(H, W).total;
    default: return packed_layout<float>(H, W).total;
  }
}

int auto_rows_dev(int H, int W) {
  const long long chunks = ((long long)(W / FD_DEV_VEC) + kDevLanes - 1) / kDevLanes;
  long long R = (long long)H * chunks / (152LL * 64);
  if (R < 4) R = 4;
  if (R > 64) R = 64;
  if (R > H) R = H;
  return (int)R;
}

}  // namespace
}  // namespace fd

using namespace fd;

extern "C" {

size_t fd_packed_bytes(int H, int W, const fd_storage* st) {
  if (H <= 0 || W <= 0 || check_storage(st) != FD_OK) return 0;
  return packed_bytes(H, W, st->dtype);
}

int fd_pack(const fd_params* prm, int src_dtype, const void* src, const fd_storage* st, void* dst, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_storage(st)) return r;
  FD_REQUIRE(src_dtype == FD_F64 || src_dtype == FD_F32, FD_ERR_DTYPE, "fd_pack: source dtype %d", src_dtype);
  FD_REQUIRE(src && dst, FD_ERR_ARG, "fd_pack: NULL pointer");
  const DevCoef c = make_dev_coef(*prm, st->f_scale_log2, st->g_scale_log2);
  cudaStream_t s = as_stream(stream);
  int r;
  if (src_dtype == FD_F64) {
    r = st->dtype == FD_F16    ? launch_pack<double, __half>(*prm, c, src, (char*)dst, s)
        : st->dtype == FD_BF16 ? launch_pack<double, __nv_bfloat16>(*prm, c, src, (char*)dst, s)
                               : launch_pack<double, float>(*prm, c, src, (char*)dst, s);
  } else {
    r = st->dtype == FD_F16    ? launch_pack<float, __half>(*prm, c, src, (char*)dst, s)
        : st->dtype == FD_BF16 ? launch_pack<float, __nv_bfloat16>(*prm, c, src, (char*)dst, s)
                               : launch_pack<float, float>(*prm, c, src, (char*)dst, s);
  }
  return r == FD_OK ? FD_OK : check_launch("fd_pack");
}

int fd_unpack(const fd_params* prm, const fd_storage* st, const void* src, int dst_dtype, void* dst, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_storage(st)) return r;
  FD_REQUIRE(dst_dtype == FD_F64 || dst_dtype == FD_F32, FD_ERR_DTYPE, "fd_unpack: destination dtype %d", dst_dtype);
  FD_REQUIRE(src && dst, FD_ERR_ARG, "fd_unpack: NULL pointer");
  const DevCoef c = make_dev_coef(*prm, st->f_scale_log2, st->g_scale_log2);
  cudaStream_t s = as_stream(stream);
  int r;
  if (dst_dtype == FD_F64) {
    r = st->dtype == FD_F16    ? launch_unpack<double, __half>(*prm, c, (const char*)src, dst, s)
        : st->dtype == FD_BF16 ? launch_unpack<double, __nv_bfloat16>(*prm, c, (const char*)src, dst, s)
                               : launch_unpack<double, float>(*prm, c, (const char*)src, dst, s);
  } else {
    r = st->dtype == FD_F16    ? launch_unpack<float, __half>(*prm, c, (const char*)src, dst, s)
        : st->dtype == FD_BF16 ? launch_unpack<float, __nv_bfloat16>(*prm, c, (const char*)src, dst, s)
                               : launch_unpack<float, float>(*prm, c, (const char*)src, dst, s);
  }
  return r == FD_OK ? FD_OK : check_launch("fd_unpack");
}

int fd_fused_step_packed(const fd_params* prm, const fd_storage* st, const uint16_t* mask, const double* inlet_ux,
                         void* pop_a, void* pop_b, void* side_a, void* side_b, int nsteps, int rows_per_warp,
                         void* stream) {
  if (int r = check_params(prm)) return r;
  FD_REQUIRE(prm->variant != FD_VARIANT_PERIODIC_XY, FD_ERR_SHAPE,
             "fd_fused_step_packed: the periodic-xy body-force variant runs on the reference-order kernels "
             "(fd_fused_step, FP64 / FP32) only");
  if (int r = check_storage(st)) return r;
  FD_REQUIRE(mask && inlet_ux && pop_a && pop_b && side_a && side_b, FD_ERR_ARG, "fd_fused_step_packed: NULL pointer");
  FD_REQUIRE(pop_a != pop_b && side_a != side_b, FD_ERR_ARG, "fd_fused_step_packed: ping-pong buffers must differ");
  FD_REQUIRE(nsteps >= 0, FD_ERR_ARG, "fd_fused_step_packed: negative step count");
  const int vec = FD_DEV_VEC;
  FD_REQUIRE(prm->W % 4 == 0 && prm->W >= 2 * vec && prm->H >= 3, FD_ERR_SHAPE,
             "fd_fused_step_packed: W must be a multiple of 4 and >= %d, H >= 3 (got %dx%d)", 2 * vec, prm->H, prm->W);
  FD_REQUIRE(((uintptr_t)pop_a | (uintptr_t)pop_b) % 256 == 0 && (uintptr_t)mask % 16 == 0, FD_ERR_ARG,
             "fd_fused_step_packed: population buffers must be 256-byte aligned");
  if (nsteps == 0) return FD_OK;
  const DevCoef c = make_dev_coef(*prm, st->f_scale_log2, st->g_scale_log2);
  cudaStream_t s = as_stream(stream);
  // shared-memory staged kernel: needs 16-byte aligned rows of every plane
  if (prm->W % 8 == 0) {
    const int r = fused_tma(*prm, *st, c, mask, inlet_ux, pop_a, pop_b, side_a, side_b, nsteps, rows_per_warp, s);
    return r == FD_OK ? FD_OK : check_launch("fd_fused_step_packed");
  }
  const int R = rows_per_warp > 0 ? rows_per_warp : auto_rows_dev(prm->H, prm->W);
  float* sa = (float*)side_a;
  float* sb = (float*)side_b;
  const bool sr = st->rounding == FD_ROUND_STOCHASTIC;
  char* pa = (char*)pop_a;
  char* pb = (char*)pop_b;
  int r;
  switch (st->dtype) {
    case FD_F16:
      r = sr ? launch_fused_dev<__half, FD_DEV_VEC, true>(*prm, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R, st->seed, s)
             : launch_fused_dev<__half, FD_DEV_VEC, false>(*prm, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R, 0, s);
      break;
    case FD_BF16:
      r = sr ? launch_fused_dev<__nv_bfloat16, FD_DEV_VEC, true>(*prm, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R,
                                                                 st->seed, s)
             : launch_fused_dev<__nv_bfloat16, FD_DEV_VEC, false>(*prm, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R, 0,
                                                                  s);
      break;
    default:
      r = launch_fused_dev<float, FD_DEV_VEC, false>(*prm, c, mask, inlet_ux, pa, pb, sa, sb, nsteps, R, 0, s);
  }
  return r == FD_OK ? FD_OK : check_launch("fd_fused_step_packed");
}

}  // extern "C"
