// Shared device definitions for the two-phase D2Q9 lattice-Boltzmann kernels.
//
// Layout conventions (all kernels):
//   populations  f, g : direction-major structure of arrays, plane i at
//                       base + i*H*W, row-major (y, x) inside a plane
//                       (the reference's (9, H, W) arrays, fingering_periodic.py:107-108)
//   fields             : (H, W) row-major
//   mask word          : uint16 per cell; bits 0..7 bounce-back link of
//                        populations 1..8, bit 8 solid
//   side arrays        : 6 x H values [gx(x=0), gy(x=0), mu(x=0), gx(x=W-1), gy(x=W-1), mu(x=W-1)]
//                        - the psi derivatives and mu the Zou-He rules read
//                        (fingering_periodic.py:273-275, 309-311)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/fdlbm.h"

namespace fd {

// D2Q9 velocity set and weights (fingering_periodic.py:50-89)
__host__ __device__ constexpr int ex_of(int i) { return (i == 1 || i == 5 || i == 8) ? 1 : (i == 3 || i == 6 || i == 7) ? -1 : 0; }
__host__ __device__ constexpr int ey_of(int i) { return (i == 2 || i == 5 || i == 6) ? 1 : (i == 4 || i == 7 || i == 8) ? -1 : 0; }
__host__ __device__ constexpr int opp_of(int i) { return i == 0 ? 0 : (i <= 4 ? ((i + 1) % 4) + 1 : ((i - 3) % 4) + 5); }
static_assert(opp_of(1) == 3 && opp_of(2) == 4 && opp_of(3) == 1 && opp_of(4) == 2, "opp");
static_assert(opp_of(5) == 7 && opp_of(6) == 8 && opp_of(7) == 5 && opp_of(8) == 6, "opp");

constexpr uint16_t SOLID = 1u << 8;

// Coefficients in the compute type T.  Every entry is evaluated on the host
// in double precision with the reference's operand order and then rounded
// to T, so the FP64 kernels see the exact constants the reference sees.
template <typename T>
struct Coef {
  T w[9];
  T tau_inv;     // 1.0 / tau                      (fingering_periodic.py:263)
  T eta_n;       // Eta_n                          (fingering_periodic.py:203)
  T eta_n_M;     // Eta_n * M                      (fingering_periodic.py:204)
  T a, kappa;    //                                (fingering_periodic.py:143)
  T c_a0;        // 3.0 * (1.0 - w0)               (fingering_periodic.py:156)
  T c_b0;        // 3.0 * (1.0 - w0) * gamma       (fingering_periodic.py:164)
  T c_b18;       // 3 * gamma                      (fingering_periodic.py:168)
  T psi_wall;
  T one_third;   // 1 / 3                          (fingering_periodic.py:124)
  T two_thirds;  // 2 / 3                          (fingering_periodic.py:283)
  T one_sixth;   // 1.0 / 6.0                      (fingering_periodic.py:287)
  T out_coef;    // 2/3 (fingering_periodic.py:317) or 1.5 (fingering.py:378)
  T wsum_in;     // w1 + w5 + w8
  T wsum_out;    // w3 + w6 + w7
  T wsum_68;     // w6 + w8                        (fingering.py:346)
  T wsum_57;     // w5 + w7                        (fingering.py:362)
  T bx, by;      // body force per unit mass (FD_VARIANT_PERIODIC_XY; no reference counterpart)
  int body;      // 1: add the body force to the velocity and the forcing term
  int p_out;     // 1: pressure outlet rho = 1 (FD_OUTLET_PRESSURE; no reference counterpart)
};

template <typename T>
inline Coef<T> make_coef(const fd_params& p) {
  const double w[9] = {4.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
  Coef<T> c;
  for (int i = 0; i < 9; ++i) c.w[i] = (T)w[i];
  c.tau_inv = (T)(1.0 / p.tau);
  c.eta_n = (T)p.eta_n;
  c.eta_n_M = (T)(p.eta_n * p.M);
  c.a = (T)p.a;
  c.kappa = (T)p.kappa;
  const double ca0 = 3.0 * (1.0 - w[0]);
  c.c_a0 = (T)ca0;
  c.c_b0 = (T)(ca0 * p.gamma);
  c.c_b18 = (T)(3 * p.gamma);
  c.psi_wall = (T)p.psi_wall;
  c.one_third = (T)(1.0 / 3.0);
  c.two_thirds = (T)(2.0 / 3.0);
  c.one_sixth = (T)(1.0 / 6.0);
  c.out_coef = (T)p.outlet_coef;
  c.wsum_in = (T)((w[1] + w[5]) + w[8]);
  c.wsum_out = (T)((w[3] + w[6]) + w[7]);
  c.wsum_68 = (T)(w[6] + w[8]);
  c.wsum_57 = (T)(w[5] + w[7]);
  c.body = p.variant == FD_VARIANT_PERIODIC_XY;
  c.bx = (T)(c.body ? p.force_x : 0.0);
  c.by = (T)(c.body ? p.force_y : 0.0);
  c.p_out = (p.flags & FD_OUTLET_PRESSURE) ? 1 : 0;
  return c;
}

// ---------------------------------------------------------------------------
// vector global memory access (aligned, VEC elements of S)
// ---------------------------------------------------------------------------
template <typename S, int VEC>
__device__ __forceinline__ void ld_vec(const S* __restrict__ p, S (&v)[VEC]) {
  constexpr int B = (int)sizeof(S) * VEC;
  static_assert(B == 4 || B == 8 || B == 16 || B == 32, "vector width");
  if constexpr (B == 32) {
    uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
    uint4 b = __ldg(reinterpret_cast<const uint4*>(p) + 1);
    memcpy(&v[0], &a, 16);
    memcpy(reinterpret_cast<char*>(&v[0]) + 16, &b, 16);
  } else if constexpr (B == 16) {
    uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
    memcpy(&v[0], &a, 16);
  } else if constexpr (B == 8) {
    uint2 a = __ldg(reinterpret_cast<const uint2*>(p));
    memcpy(&v[0], &a, 8);
  } else {
    unsigned a = __ldg(reinterpret_cast<const unsigned*>(p));
    memcpy(&v[0], &a, 4);
  }
}

template <typename S, int VEC>
__device__ __forceinline__ void st_vec(S* __restrict__ p, const S (&v)[VEC]) {
  constexpr int B = (int)sizeof(S) * VEC;
  if constexpr (B == 32) {
    uint4 a, b;
    memcpy(&a, &v[0], 16);
    memcpy(&b, reinterpret_cast<const char*>(&v[0]) + 16, 16);
    reinterpret_cast<uint4*>(p)[0] = a;
    reinterpret_cast<uint4*>(p)[1] = b;
  } else if constexpr (B == 16) {
    uint4 a;
    memcpy(&a, &v[0], 16);
    *reinterpret_cast<uint4*>(p) = a;
  } else if constexpr (B == 8) {
    uint2 a;
    memcpy(&a, &v[0], 8);
    *reinterpret_cast<uint2*>(p) = a;
  } else {
    unsigned a;
    memcpy(&a, &v[0], 4);
    *reinterpret_cast<unsigned*>(p) = a;
  }
}

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

}  // namespace fd
