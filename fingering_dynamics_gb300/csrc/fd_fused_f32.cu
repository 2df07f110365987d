// FP32 instantiation of the fused step (storage and arithmetic in FP32,
// contraction to FMA allowed).
#include "fd_fused.cuh"

namespace fd {
int fused_f32(const fd_params& p, const uint16_t* mask, const double* inlet_ux, void* pa, void* pb, void* sa, void* sb,
              int nsteps, int R, cudaStream_t st) {
  return launch_fused<float, 4>(p, mask, inlet_ux, (float*)pa, (float*)pb, (float*)sa, (float*)sb, nsteps, R, st);
}
}  // namespace fd
