// Fused step: one kernel per iteration of the reference's loop body.
//
// State between kernels: the post-collision populations of iteration n-1
// (f planes 0..8, g planes 9..17) plus the side arrays (psi_x, psi_y, mu at
// columns 0 and W-1) of iteration n-1.  One kernel
//   1. pulls the state (stream, fingering_periodic.py:327-343), applies the
//      bounce-back link bits (bounce_back.py, fingering.py:573) and the
//      Zou-He rules of iteration n-1 (fingering_periodic.py:268-324),
//   2. forms psi = sum g (fingering_periodic.py:210-212) on its rows and one
//      halo row/column each side, the psi stencils, mu, u, p, tau_mix
//      (fingering_periodic.py:472-479),
//   3. collides (fingering_periodic.py:455-460) and writes the new state and
//      the new side arrays.
//
// Work decomposition: a warp owns a strip of 30*VEC consecutive cells of a
// row band (lanes 1..30, VEC cells per lane, 16-byte vector accesses) and
// marches down R rows.  Lanes 0 and 31 are halo lanes: they load the
// neighbouring vectors so that x-shifted populations and the psi of the
// cells left and right of the strip come from warp shuffles, and they store
// nothing.  psi of the rows above and below travels in registers as the
// warp marches, so each population is read from HBM once per step (plus two
// halo rows of g per strip) and written once.
#pragma once

#include "fd_zouhe.cuh"

namespace fd {

constexpr int kFusedLanes = 30;  // owned vectors per warp-row

template <typename T>
struct FusedArgs {
  Coef<T> c;
  int H, W, variant, nchunks, nstrips, R;
  const uint16_t* __restrict__ mask;
  const double* __restrict__ inlet_ux;
  const T* __restrict__ src;   // 18 planes
  T* __restrict__ dst;         // 18 planes
  const T* __restrict__ side_in;
  T* __restrict__ side_out;
};

// Raw pull of one row of 9 planes: out[i][k] = plane_i(x0 + k - ex_i, y - ey_i),
// periodic in x and y; then bounce-back links of the row's cells.
template <typename T, int VEC>
__device__ __forceinline__ void pull_row(const T* __restrict__ planes, size_t P, int H, int W, int y, int xw,
                                         const uint16_t (&mb)[VEC], T (&out)[9][VEC]) {
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int ex = ex_of(i), ey = ey_of(i);
    const int ys = wrap(y - ey, H);
    T v[VEC];
    ld_vec<T, VEC>(planes + (size_t)i * P + (size_t)ys * W + xw, v);
    if (ex == 0) {
#pragma unroll
      for (int k = 0; k < VEC; ++k) out[i][k] = v[k];
    } else if (ex == 1) {
      const T l = __shfl_up_sync(0xffffffffu, v[VEC - 1], 1);
      out[i][0] = l;
#pragma unroll
      for (int k = 1; k < VEC; ++k) out[i][k] = v[k - 1];
    } else {
      const T r = __shfl_down_sync(0xffffffffu, v[0], 1);
#pragma unroll
      for (int k = 0; k < VEC - 1; ++k) out[i][k] = v[k + 1];
      out[i][VEC - 1] = r;
    }
  }
  // half-way bounce-back: the post-collision opposite population of the same cell
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    const unsigned bits = mb[k] & 0xFFu;
    if (bits) {
      const size_t q = (size_t)y * W + xw + k;
#pragma unroll
      for (int i = 1; i < 9; ++i)
        if (bits & (1u << (i - 1))) out[i][k] = planes[(size_t)opp_of(i) * P + q];
    }
  }
}

// Single pulled population of one cell (used for the rho_inlet of rows 1 and
// H-2 that the walled variant's inlet corners read).
template <typename T>
__device__ __forceinline__ T pull_one(const T* __restrict__ planes, const uint16_t* __restrict__ mask, size_t P,
                                      int H, int W, int x, int y, int i) {
  const size_t q = (size_t)y * W + x;
  if (i > 0 && ((mask[q] >> (i - 1)) & 1u)) return planes[(size_t)opp_of(i) * P + q];
  return planes[(size_t)i * P + (size_t)wrap(y - ey_of(i), H) * W + wrap(x - ex_of(i), W)];
}

template <typename T>
__device__ __forceinline__ T rho_inlet_row(const FusedArgs<T>& a, size_t P, int yn) {
  T fn[9];
  const int dirs[6] = {0, 2, 4, 3, 6, 7};
#pragma unroll
  for (int d = 0; d < 6; ++d) fn[dirs[d]] = pull_one(a.src, a.mask, P, a.H, a.W, 0, yn, dirs[d]);
  fn[1] = fn[5] = fn[8] = T(0);
  return inlet_rho(fn, (T)a.inlet_ux[yn], a.side_in[0 * a.H + yn], a.side_in[2 * a.H + yn]);
}

// psi of a pulled row (x ghosts +1 / -1, psi_wall on solid cells; the
// halo lanes' wrapped cells for FD_VARIANT_PERIODIC_XY)
template <typename T, int VEC>
__device__ __forceinline__ void psi_row(const FusedArgs<T>& a, int x0, const uint16_t (&mb)[VEC],
                                        const T (&g)[9][VEC], T (&psi)[VEC]) {
  const bool ghosts = a.variant != FD_VARIANT_PERIODIC_XY;
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    const int x = x0 + k;
    T s = g[0][k];
#pragma unroll
    for (int i = 1; i < 9; ++i) s = s + g[i][k];
    psi[k] = (ghosts && x < 0) ? T(1) : (ghosts && x >= a.W) ? T(-1) : ((mb[k] & SOLID) ? a.c.psi_wall : s);
  }
}

// Pull g of row y (wrapped for the periodic variant) with Zou-He, and its psi.
template <typename T, int VEC>
__device__ __forceinline__ void g_row(const FusedArgs<T>& a, size_t P, int y, int x0, int xw, uint16_t (&mb)[VEC],
                                      T (&g)[9][VEC], T (&psi)[VEC]) {
  ld_vec<uint16_t, VEC>(a.mask + (size_t)y * a.W + xw, mb);
  pull_row<T, VEC>(a.src + 9 * P, P, a.H, a.W, y, xw, mb, g);
  if (x0 == 0) {
    T gc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gc[i] = g[i][0];
    zou_he_g(a.c, a.variant, a.H, a.W, 0, y, gc);
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i][0] = gc[i];
  }
  if (x0 == a.W - VEC) {
    T gc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gc[i] = g[i][VEC - 1];
    zou_he_g(a.c, a.variant, a.H, a.W, a.W - 1, y, gc);
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i][VEC - 1] = gc[i];
  }
  psi_row<T, VEC>(a, x0, mb, g, psi);
}

// Zou-He on the f populations of element K (a cell of column 0 or W-1) and
// the side values of this iteration for the next kernel.
template <typename T, int VEC, int K>
__device__ __forceinline__ void boundary_cell(const FusedArgs<T>& a, size_t P, int y, int x, T (&f)[9][VEC],
                                              const T (&gx)[VEC], const T (&gy)[VEC], const T (&lap)[VEC],
                                              const T (&Pc)[VEC]) {
  const int o = (x == 0) ? 0 : 3;
  T rho_nb = T(0);
  if (a.variant == FD_VARIANT_WALLS && x == 0 && (y == 0 || y == a.H - 1))
    rho_nb = rho_inlet_row(a, P, y == 0 ? 1 : a.H - 2);
  T fc[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) fc[i] = f[i][K];
  zou_he_f(a.c, a.variant, a.H, a.W, x, y, fc, (T)a.inlet_ux[y], a.side_in[(o + 0) * a.H + y],
           a.side_in[(o + 1) * a.H + y], a.side_in[(o + 2) * a.H + y], rho_nb);
#pragma unroll
  for (int i = 0; i < 9; ++i) f[i][K] = fc[i];
  // getMu_plain of this iteration's psi and laplacian (fingering_periodic.py:146-149)
  a.side_out[(o + 0) * a.H + y] = gx[K];
  a.side_out[(o + 1) * a.H + y] = gy[K];
  a.side_out[(o + 2) * a.H + y] = chem_pot(a.c, Pc[K], lap[K]);
}

template <typename T, int VEC>
__device__ __forceinline__ void extend(const T (&p)[VEC], T (&e)[VEC + 2]) {
  e[0] = __shfl_up_sync(0xffffffffu, p[VEC - 1], 1);
#pragma unroll
  for (int k = 0; k < VEC; ++k) e[k + 1] = p[k];
  e[VEC + 1] = __shfl_down_sync(0xffffffffu, p[0], 1);
}

#ifndef FD_FUSED_MINB
#define FD_FUSED_MINB 1
#endif

template <typename T, int VEC>
__global__ void __launch_bounds__(128, FD_FUSED_MINB) k_fused_step(const FusedArgs<T> a) {
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (warp >= a.nchunks * a.nstrips) return;  // warp-uniform
  const int chunk = warp % a.nchunks, strip = warp / a.nchunks;
  const int x0 = (chunk * kFusedLanes + lane - 1) * VEC;
  const int xw = ((x0 % a.W) + a.W) % a.W;
  const bool owned = lane >= 1 && lane <= kFusedLanes && x0 >= 0 && x0 < a.W;
  const int y0 = strip * a.R, y1 = min(y0 + a.R, a.H);
  const size_t P = (size_t)a.H * a.W;
  const bool walls = a.variant == FD_VARIANT_WALLS;

  T gC[9][VEC], gN[9][VEC];
  T Pm[VEC], Pc[VEC], Pn[VEC];
  uint16_t mC[VEC], mN[VEC];

  // psi of the row above the strip (y0 - 1)
  if (walls && y0 == 0) {
#pragma unroll
    for (int k = 0; k < VEC; ++k) Pm[k] = a.c.psi_wall;
  } else {
    g_row<T, VEC>(a, P, wrap(y0 - 1, a.H), x0, xw, mN, gN, Pm);
  }
  g_row<T, VEC>(a, P, y0, x0, xw, mC, gC, Pc);

  for (int y = y0; y < y1; ++y) {
    // row y+1: pulled g and psi (ghost psi_wall row past the top wall)
    if (walls && y + 1 >= a.H) {
#pragma unroll
      for (int k = 0; k < VEC; ++k) Pn[k] = a.c.psi_wall;
    } else {
      g_row<T, VEC>(a, P, wrap(y + 1, a.H), x0, xw, mN, gN, Pn);
    }

    // psi stencils of row y
    T em[VEC + 2], ec[VEC + 2], en[VEC + 2];
    extend<T, VEC>(Pm, em);
    extend<T, VEC>(Pc, ec);
    extend<T, VEC>(Pn, en);
    T gx[VEC], gy[VEC], lap[VEC];
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
      gx[k] = grad_x(ec[k + 2], ec[k], en[k + 2], en[k], em[k + 2], em[k]);
      gy[k] = grad_y(en[k + 1], em[k + 1], en[k + 2], en[k], em[k + 2], em[k]);
      lap[k] = laplacian(ec[k + 1], ec[k + 2], ec[k], en[k + 1], em[k + 1], en[k + 2], en[k], em[k + 2], em[k]);
    }

    // f of row y: pull, bounce-back, Zou-He with the previous iteration's side values
    T f[9][VEC];
    pull_row<T, VEC>(a.src, P, a.H, a.W, y, xw, mC, f);
    if (owned && x0 == 0) boundary_cell<T, VEC, 0>(a, P, y, 0, f, gx, gy, lap, Pc);
    if (owned && x0 == a.W - VEC) boundary_cell<T, VEC, VEC - 1>(a, P, y, a.W - 1, f, gx, gy, lap, Pc);

    // macroscopic fields and collision on fluid cells
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
      if (!(mC[k] & SOLID)) {
        T fc[9], gc[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) { fc[i] = f[i][k]; gc[i] = gC[i][k]; }
        const Macro<T> m = macros_of(a.c, fc, Pc[k], gx[k], gy[k], lap[k]);
        collide(a.c, m, fc, gc);
#pragma unroll
        for (int i = 0; i < 9; ++i) { f[i][k] = fc[i]; gC[i][k] = gc[i]; }
      }
    }
    if (owned) {
      const size_t row = (size_t)y * a.W + x0;
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        st_vec<T, VEC>(a.dst + (size_t)i * P + row, f[i]);
        st_vec<T, VEC>(a.dst + (size_t)(9 + i) * P + row, gC[i]);
      }
    }
    // march
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
      Pm[k] = Pc[k];
      Pc[k] = Pn[k];
      mC[k] = mN[k];
#pragma unroll
      for (int i = 0; i < 9; ++i) gC[i][k] = gN[i][k];
    }
  }
}

template <typename T, int VEC>
int launch_fused(const fd_params& p, const uint16_t* mask, const double* inlet_ux, T* pa, T* pb, T* sa, T* sb,
                 int nsteps, int R, cudaStream_t st) {
  FusedArgs<T> a;
  a.c = make_coef<T>(p);
  a.H = p.H;
  a.W = p.W;
  a.variant = p.variant;
  const int nvec = p.W / VEC;
  a.nchunks = (nvec + kFusedLanes - 1) / kFusedLanes;
  a.R = R;
  a.nstrips = (p.H + R - 1) / R;
  a.mask = mask;
  a.inlet_ux = inlet_ux;
  const long long warps = (long long)a.nchunks * a.nstrips;
  const unsigned blocks = (unsigned)((warps * 32 + 127) / 128);
  for (int s = 0; s < nsteps; ++s) {
    const bool even = (s % 2) == 0;
    a.src = even ? pa : pb;
    a.dst = even ? pb : pa;
    a.side_in = even ? sa : sb;
    a.side_out = even ? sb : sa;
    k_fused_step<T, VEC><<<blocks, 128, 0, st>>>(a);
  }
  return cudaGetLastError() == cudaSuccess ? FD_OK : FD_ERR_CUDA;
}

}  // namespace fd
