// FP32 instantiation of the fused step (storage and arithmetic in FP32,
// contraction to FMA allowed).
#include "fd_fused.cuh"

#ifndef FD_F32_VEC
#define FD_F32_VEC 4
#endif

namespace fd {
int fused_f32(const fd_params& p, const uint16_t* mask, const double* inlet_ux, void* pa, void* pb, void* sa, void* sb,
              int nsteps, int R, cudaStream_t st) {
  return launch_fused<float, FD_F32_VEC>(p, mask, inlet_ux, (float*)pa, (float*)pb, (float*)sa, (float*)sb, nsteps, R, st);
}
}  // namespace fd
