// FP64 instantiation of the fused step.  Built with -fmad=false: the per-cell
// arithmetic is the reference's operand order without contraction, so the
// fused FP64 step equals the reference-order kernels (and the reference) bit
// for bit.
#include "fd_fused.cuh"

namespace fd {
int fused_f64(const fd_params& p, const uint16_t* mask, const double* inlet_ux, void* pa, void* pb, void* sa, void* sb,
              int nsteps, int R, cudaStream_t st) {
  return launch_fused<double, 2>(p, mask, inlet_ux, (double*)pa, (double*)pb, (double*)sa, (double*)sb, nsteps, R, st);
}
}  // namespace fd
