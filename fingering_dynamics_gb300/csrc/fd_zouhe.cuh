// Zou-He boundary application per cell, shared by the per-function kernels
// and the fused step.  `x`, `y` are the cell; `f`/`g` its post-stream,
// post-bounce-back populations; `side` values (gx, gy, mu) are those of the
// previous iteration's psi (fingering_periodic.py:273-275 runs before psi is
// updated at fingering_periodic.py:471).
#pragma once

#include "fd_physics.cuh"

namespace fd {

// g part of zou_he_boundary_inlet/outlet at one cell.
template <typename T>
__device__ __forceinline__ void zou_he_g(const Coef<T>& c, int variant, int H, int W, int x, int y, T (&g)[9]) {
  if (variant == FD_VARIANT_PERIODIC_XY) return;  // no inlet / outlet
  if (x == 0) {
    if (variant == FD_VARIANT_WALLS) {
      if (y == 0) inlet_corner_bottom_g(c, g);
      else if (y == H - 1) inlet_corner_top_g(c, g);
      else inlet_g(c, g);
    } else {
      inlet_g(c, g);
    }
  }
  if (x == W - 1) {
    outlet_g(c, g);
    if (variant == FD_VARIANT_WALLS) {
      if (y == 0) g[2] = g[4];          // fingering.py:388
      if (y == H - 1) g[4] = g[2];      // fingering.py:390
    }
  }
}

// f part at one cell of column 0 or W-1.  gx, gy, mu are the side values of
// that column and row; rho_nb is rho_inlet of row 1 (for y == 0) or of row
// H-2 (for y == H-1) in the walled variant, unused otherwise.
template <typename T>
__device__ __forceinline__ void zou_he_f(const Coef<T>& c, int variant, int H, int W, int x, int y, T (&f)[9],
                                         T ux, T gx, T gy, T mu, T rho_nb) {
  if (variant == FD_VARIANT_PERIODIC_XY) return;  // no inlet / outlet
  if (x == 0) {
    if (variant == FD_VARIANT_WALLS && y == 0) inlet_corner_bottom_f(f, rho_nb);
    else if (variant == FD_VARIANT_WALLS && y == H - 1) inlet_corner_top_f(f, rho_nb);
    else inlet_f(c, f, ux, gx, gy, mu);
  }
  if (x == W - 1) {
    outlet_f(c, f, ux, gx, gy, mu);
    if (variant == FD_VARIANT_WALLS) {
      if (y == 0) f[2] = f[4];          // fingering.py:387
      if (y == H - 1) f[4] = f[2];      // fingering.py:389
    }
  }
}

}  // namespace fd
