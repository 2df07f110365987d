// Deviation-form physics for the FP32-compute fused kernels.
//
// The f populations are carried as deviations d_i = f_i - w_i from the rest
// state rho = 1, u = 0 (optionally scaled and stored in FP16/BF16); g is
// carried as is, with g_0 (which holds most of psi) always in FP32.  The
// model is the reference's (fingering_periodic.py:123-264), rewritten so that
// every quantity that is small is computed from small quantities:
//
//   rho = 1 + sum d_i                      j = sum d_i e_i
//   3p - 1 = (rho - 1) + 3 psi mu          (getP, fingering_periodic.py:123-124)
//   feq_0 - w_0 = w_0 (rho-1) - 3(1-w_0) psi mu + w_0 rho q_0
//   feq_i - w_i = w_i ((rho-1) + 3 psi mu + rho q_i)          i >= 1
//   geq_0 - g_0 = (sum_{i>=1} g_i) - 3(1-w_0) gamma mu + w_0 psi q_0
//   geq_i       = w_i (3 gamma mu + psi q_i)                   i >= 1
//   F_i = mu (1 - 1/(2 tau)) w_i [3 e_i.grad psi - 3 u.grad psi + 9 (e_i.u)(e_i.grad psi)]
//   1/tau_mix = rho D / (6 eta1 eta2 + rho D / 2),  D = (eta1 + eta2) + (eta2 - eta1) psi
//
// with q_i = 3 e_i.u + 4.5 (e_i.u)^2 - 1.5 u^2, eta1 = Eta_n, eta2 = M Eta_n.
// These are algebraically identical to the reference's expressions (the
// mixing rule of fingering_periodic.py:201-208 is multiplied through, so the
// reference's tau pole at D = 0 becomes 1/tau = 0).  The Zou-He rules
// (fingering_periodic.py:268-324, fingering.py:298-390) carry over to
// deviations because the weights they pair are equal (w1 = w3, w2 = w4,
// w5 = w7, w6 = w8) and their weight sums are 1 or 17/18.
#pragma once

#include <cuda_bf16.h>
#include <type_traits>
#include <cuda_fp16.h>

#include "fd_common.cuh"

namespace fd {

struct DevCoef {
  float w[9];
  float inv_tau_g;     // 1 / tau
  float eta_sum;       // eta1 + eta2
  float eta_diff;      // eta2 - eta1
  float six_eta_prod;  // 6 eta1 eta2
  float a, kappa;
  float c_b0;          // 3 (1 - w0) gamma
  float three_gamma;   // 3 gamma
  float c_a0;          // 3 (1 - w0)
  float psi_wall;
  float out_coef;      // 2/3 or 1.5
  float sf, inv_sf;    // storage scale of f deviations
  float sg, inv_sg;    // storage scale of g_1..g_8
  int p_out;           // pressure outlet rho = 1 (FD_OUTLET_PRESSURE)
};

inline DevCoef make_dev_coef(const fd_params& p, int f_scale_log2, int g_scale_log2) {
  const double w[9] = {4.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
  DevCoef c;
  for (int i = 0; i < 9; ++i) c.w[i] = (float)w[i];
  const double e1 = p.eta_n, e2 = p.eta_n * p.M;
  c.inv_tau_g = (float)(1.0 / p.tau);
  c.eta_sum = (float)(e1 + e2);
  c.eta_diff = (float)(e2 - e1);
  c.six_eta_prod = (float)(6.0 * e1 * e2);
  c.a = (float)p.a;
  c.kappa = (float)p.kappa;
  c.c_b0 = (float)(3.0 * (1.0 - w[0]) * p.gamma);
  c.three_gamma = (float)(3.0 * p.gamma);
  c.c_a0 = (float)(3.0 * (1.0 - w[0]));
  c.psi_wall = (float)p.psi_wall;
  c.out_coef = (float)p.outlet_coef;
  c.sf = ldexpf(1.0f, f_scale_log2);
  c.inv_sf = ldexpf(1.0f, -f_scale_log2);
  c.sg = ldexpf(1.0f, g_scale_log2);
  c.inv_sg = ldexpf(1.0f, -g_scale_log2);
  c.p_out = (p.flags & FD_OUTLET_PRESSURE) ? 1 : 0;
  return c;
}

// ---- storage conversion -----------------------------------------------------
template <typename S> __device__ __forceinline__ float to_f(S v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<__half>(__half v) { return __half2float(v); }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename S> __device__ __forceinline__ S from_f(float v);
template <> __device__ __forceinline__ float from_f<float>(float v) { return v; }
template <> __device__ __forceinline__ __half from_f<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// ---- stochastic rounding ----------------------------------------------------
// Counter-based randomness: a 32-bit integer hash (the "lowbias32" xorshift-
// multiply construction, constants from its published parameter search) of
// the cell index mixed with the step's seed, then a 32-bit linear congruential
// sequence (Numerical Recipes' constants) for the successive stores of a
// cell; only the high bits of each value are used.
__host__ __device__ __forceinline__ uint32_t sr_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
__device__ __forceinline__ uint32_t sr_next(uint32_t s) { return s * 1664525u + 1013904223u; }

// FP32 -> storage type, rounding the magnitude up with probability equal to
// the discarded fraction: add uniform random bits below the last kept bit of
// the FP32 pattern, then truncate.  (Below the FP16 normal range, 6.1e-5, more
// bits are discarded than dithered: there the rounding leans towards zero by
// at most one FP16 subnormal step, 6e-8.)
// Two values to the storage type in one conversion: the 32-bit word holds lo in
// its low half and hi in its high half (cvt.rn / cvt.rs .f16x2 / .bf16x2; the
// stochastic form rounds each value up with probability equal to its discarded
// fraction, from the 32 random bits r, different bits for the two values).
template <typename S> __device__ __forceinline__ uint32_t pair_from_f(float lo, float hi);
template <> __device__ __forceinline__ uint32_t pair_from_f<__half>(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}
template <> __device__ __forceinline__ uint32_t pair_from_f<__nv_bfloat16>(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}
template <typename S> __device__ __forceinline__ uint32_t pair_from_f_sr(float lo, float hi, uint32_t r);
template <> __device__ __forceinline__ uint32_t pair_from_f_sr<__half>(float lo, float hi, uint32_t r) {
  uint32_t d;
  asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(r));
  return d;
}
template <> __device__ __forceinline__ uint32_t pair_from_f_sr<__nv_bfloat16>(float lo, float hi, uint32_t r) {
  uint32_t d;
  asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(r));
  return d;
}

template <typename S> __device__ __forceinline__ S from_f_sr(float v, uint32_t r);
template <> __device__ __forceinline__ float from_f_sr<float>(float v, uint32_t) { return v; }
template <> __device__ __forceinline__ __half from_f_sr<__half>(float v, uint32_t r) {
  return __float2half_rz(__uint_as_float(__float_as_uint(v) + (r >> 19)));
}
template <> __device__ __forceinline__ __nv_bfloat16 from_f_sr<__nv_bfloat16>(float v, uint32_t r) {
  return __float2bfloat16_rz(__uint_as_float(__float_as_uint(v) + (r >> 16)));
}

// ---- macroscopic state of one fluid cell -------------------------------------
struct DevMacro {
  float drho, rho, ux, uy, psi, mu, gx, gy, inv_tau, pref;
};

// ---- psi and its stencils -------------------------------------------------
// psi = sum of g (fingering_periodic.py:210-212) as the unevaluated sum hi + lo
// of two floats: hi = fl(g_0 + S) with S = g_1 + .. + g_8 (small), lo = the
// rounding error of that addition, exact by the TwoSum algorithm (Knuth, TAOCP
// vol. 2, 4.2.2).  Near the pure phases psi is close to +-1, where one float
// resolves it to 6e-8 only; the stencils below take differences of
// neighbouring psi values and the free energy takes 1 - psi^2, both of which
// lose that resolution to cancellation when psi is a single float.
__device__ __forceinline__ float2 dev_psi_pair(const float (&g)[9]) {
  const float S = ((g[1] + g[2]) + (g[3] + g[4])) + ((g[5] + g[6]) + (g[7] + g[8]));
  const float hi = g[0] + S;
  const float b = hi - g[0];
  const float lo = (g[0] - (hi - b)) + (S - b);
  return make_float2(hi, lo);
}

// d(psi)/dx, d(psi)/dy and the laplacian of the 3x3 neighbourhood
// (fingering_periodic.py:214-256), and the factor 1 - psi^2 of the bulk free
// energy (fingering_periodic.py:141-144).
struct DevStencil {
  float gx, gy, lap, psi, omp;
};

// Single-float psi (FP16/BF16 storage, whose own resolution is far coarser).
__device__ __forceinline__ DevStencil dev_stencil(float C, float E, float Wv, float N, float S, float NE, float NW,
                                                  float SE, float SW) {
  DevStencil s;
  s.gx = (4.0f * (E - Wv) + ((NE - NW) + (SE - SW))) * (1.0f / 12.0f);
  s.gy = (4.0f * (N - S) + ((NE - SE) + (NW - SW))) * (1.0f / 12.0f);
  s.lap = (4.0f * ((N + S) + (E + Wv)) + ((NE + NW) + (SE + SW)) - 20.0f * C) * (1.0f / 6.0f);
  s.psi = C;
  s.omp = fmaf(-C, C, 1.0f);
  return s;
}

// Paired psi (FP32 storage): every neighbour enters as its difference from the
// centre, (hi_n - hi_c) + (lo_n - lo_c), where hi_n - hi_c is exact for close
// values; 1 - psi^2 = ((1 - hi) - lo) ((1 + hi) + lo).
__device__ __forceinline__ DevStencil dev_stencil_pair(float2 C, float2 E, float2 Wv, float2 N, float2 S, float2 NE,
                                                       float2 NW, float2 SE, float2 SW) {
  auto df = [&](float2 v) { return (v.x - C.x) + (v.y - C.y); };
  const float dE = df(E), dW = df(Wv), dN = df(N), dS = df(S);
  const float dNE = df(NE), dNW = df(NW), dSE = df(SE), dSW = df(SW);
  DevStencil s;
  s.gx = (4.0f * (dE - dW) + ((dNE - dNW) + (dSE - dSW))) * (1.0f / 12.0f);
  s.gy = (4.0f * (dN - dS) + ((dNE - dSE) + (dNW - dSW))) * (1.0f / 12.0f);
  s.lap = (4.0f * ((dN + dS) + (dE + dW)) + ((dNE + dNW) + (dSE + dSW))) * (1.0f / 6.0f);
  s.psi = C.x + C.y;
  s.omp = ((1.0f - C.x) - C.y) * ((1.0f + C.x) + C.y);
  return s;
}

// getMu_plain (fingering_periodic.py:146-149) of a stencil, the Zou-He input
// stored in the boundary-value buffer
__device__ __forceinline__ float dev_mu(const DevCoef& c, const DevStencil& s) {
  return c.a * s.psi * s.omp - c.kappa * s.lap;
}

// 1 / x rounded to nearest, or (FAST) the hardware approximation (at most
// 1 ulp from it), used where the populations are stored in FP16/BF16
template <bool FAST>
__device__ __forceinline__ float dev_rcp(float x) {
  if constexpr (FAST) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  } else {
    return __frcp_rn(x);
  }
}

template <bool FAST_RCP = false>
__device__ __forceinline__ DevMacro dev_macros(const DevCoef& c, const float (&d)[9], const DevStencil& st) {
  DevMacro m;
  float jx, jy;
  if constexpr (FAST_RCP) {
    // 16-bit storage: the sums on direction pairs (1, 2) (3, 4) (5, 6) (7, 8) in packed
    // FP32x2 arithmetic, as the collision (dev_collide_x2)
    const float2 d12 = make_float2(d[1], d[2]), d34 = make_float2(d[3], d[4]);
    const float2 d56 = make_float2(d[5], d[6]), d78 = make_float2(d[7], d[8]);
    const float2 sp = __fadd2_rn(__fadd2_rn(d12, d34), __fadd2_rn(d56, d78));
    m.drho = (d[0] + sp.x) + sp.y;
    const float2 a = __ffma2_rn(d34, make_float2(-1.0f, -1.0f), d12);  // (d1 - d3, d2 - d4)
    const float2 b = __ffma2_rn(d78, make_float2(-1.0f, -1.0f), d56);  // (d5 - d7, d6 - d8)
    jx = a.x + (b.x - b.y);
    jy = a.y + (b.x + b.y);
  } else {
    m.drho = ((d[0] + d[1]) + (d[2] + d[3])) + ((d[4] + d[5]) + (d[6] + d[7])) + d[8];
    jx = ((d[1] - d[3]) + (d[5] - d[6])) + (d[8] - d[7]);
    jy = ((d[2] - d[4]) + (d[5] - d[8])) + (d[6] - d[7]);
  }
  m.rho = 1.0f + m.drho;
  const float psi = st.psi, gx = st.gx, gy = st.gy;
  m.psi = psi;
  m.gx = gx;
  m.gy = gy;
  m.mu = dev_mu(c, st);  // getMu (fingering_periodic.py:141-144)
  const float inv_rho = dev_rcp<FAST_RCP>(m.rho);
  if constexpr (FAST_RCP) {  // getUx / getUy as one pair
    const float hm = 0.5f * m.mu;
    const float2 u = __fmul2_rn(__ffma2_rn(make_float2(hm, hm), make_float2(gx, gy), make_float2(jx, jy)),
                                make_float2(inv_rho, inv_rho));
    m.ux = u.x;
    m.uy = u.y;
  } else {
    m.ux = fmaf(0.5f * m.mu, gx, jx) * inv_rho;  // getUx (fingering_periodic.py:126-132)
    m.uy = fmaf(0.5f * m.mu, gy, jy) * inv_rho;
  }
  const float rD = m.rho * fmaf(c.eta_diff, psi, c.eta_sum);
  m.inv_tau = rD * dev_rcp<FAST_RCP>(fmaf(0.5f, rD, c.six_eta_prod));  // 1 / getMix_tau
  m.pref = m.mu * fmaf(-0.5f, m.inv_tau, 1.0f);              // mu (1 - 1/(2 tau))
  return m;
}

// D2Q9 weights as compile-time constants (fingering_periodic.py:50-89)
template <int I>
__device__ __forceinline__ constexpr float wgt() {
  return I == 0 ? 4.0f / 9.0f : (I <= 4 ? 1.0f / 9.0f : 1.0f / 36.0f);
}

// e_i . v for a compile-time direction, without multiplications by 0 or +-1
template <int I>
__device__ __forceinline__ float edot(float vx, float vy) {
  constexpr int ex = ex_of(I), ey = ey_of(I);
  if constexpr (ex == 0 && ey == 0) return 0.0f;
  else if constexpr (ey == 0) return ex > 0 ? vx : -vx;
  else if constexpr (ex == 0) return ey > 0 ? vy : -vy;
  else if constexpr (ex > 0 && ey > 0) return vx + vy;
  else if constexpr (ex < 0 && ey > 0) return vy - vx;
  else if constexpr (ex < 0 && ey < 0) return -(vx + vy);
  else return vx - vy;
}

// Relaxation of one weight class (w = 1/9: axis directions, w = 1/36:
// diagonals) with the relaxation rates folded in:
//   yr = w rho / tau        xr = yr / 2          xb = w (3p - 1) / tau
//   P  = 3 w mu (1 - 1/(2 tau))                  (forcing prefactor)
//   gt = w psi / tau_g      gs = gt / 2          gc = 3 w gamma mu / tau_g
struct DevClass {
  float yr, xr, xb, P, gt, gs, gc;
};

// One pair of opposite directions (I, opp I).  With t = 3 e.u and
// s2 = t^2 - 3 u^2, q_(+-) = +-t + s2/2, so
//   (1/tau) (feq_(+-) - w) = xr s2 + xb +- yr t
//   F_(+-) = P (eg t - u.grad psi) +- P eg            (eg = e.grad psi)
//   (1/tau_g) geq_(+-) = gs s2 + gc +- gt t
// and each population relaxes as d' = (1 - 1/tau) d + [...].
template <int I>
__device__ __forceinline__ void dev_collide_pair(const DevMacro& m, const DevClass& k, float usq3, float ug, float omt,
                                                 float omg, float& dp, float& dm, float& gp, float& gm) {
  const float t = 3.0f * edot<I>(m.ux, m.uy);
  const float eg = edot<I>(m.gx, m.gy);
  const float s2 = fmaf(t, t, -usq3);
  const float B = fmaf(eg, t, -ug);
  const float Z = fmaf(k.xr, s2, fmaf(k.P, B, k.xb));
  const float V = fmaf(k.yr, t, k.P * eg);
  dp = fmaf(omt, dp, Z + V);
  dm = fmaf(omt, dm, Z - V);
  const float G = fmaf(k.gs, s2, k.gc);
  const float Gt = k.gt * t;
  gp = fmaf(omg, gp, G + Gt);
  gm = fmaf(omg, gm, G - Gt);
}

__device__ __forceinline__ void dev_collide(const DevCoef& c, const DevMacro& m, float (&d)[9], float (&g)[9]) {
  const float base = fmaf(3.0f * m.psi, m.mu, m.drho);  // 3p - 1
  const float ug = m.ux * m.gx + m.uy * m.gy;
  const float usq3 = 3.0f * (m.ux * m.ux + m.uy * m.uy);
  const float S = ((g[1] + g[2]) + (g[3] + g[4])) + ((g[5] + g[6]) + (g[7] + g[8]));
  const float itg = c.inv_tau_g;
  const float omt = 1.0f - m.inv_tau, omg = 1.0f - itg;
  // rest direction: feq_0 - w0 = w0 (rho-1) - 3 (1-w0) psi mu - (w0 rho / 2) 3 u^2,
  // F_0 = -3 w0 mu (1 - 1/(2 tau)) u.grad psi, geq_0 - g_0 = S - 3 (1-w0) gamma mu - (w0 psi / 2) 3 u^2
  {
    constexpr float w0 = wgt<0>();
    const float deq = fmaf(w0, m.drho, fmaf(-0.5f * w0 * m.rho, usq3, -c.c_a0 * m.psi * m.mu));
    const float F = -(3.0f * w0) * m.pref * ug;
    d[0] = fmaf(deq - d[0], m.inv_tau, d[0]) + F;
    const float dg = fmaf(-0.5f * w0 * m.psi, usq3, S - c.c_b0 * m.mu);
    g[0] = fmaf(dg, itg, g[0]);
  }
  DevClass a;  // w = 1/9
  a.yr = (1.0f / 9.0f) * m.inv_tau * m.rho;
  a.xr = 0.5f * a.yr;
  a.xb = (1.0f / 9.0f) * m.inv_tau * base;
  a.P = (1.0f / 3.0f) * m.pref;
  a.gt = ((1.0f / 9.0f) * itg) * m.psi;
  a.gs = 0.5f * a.gt;
  a.gc = ((1.0f / 9.0f) * itg) * c.three_gamma * m.mu;
  DevClass b;  // w = 1/36 = (1/9) / 4
  b.yr = 0.25f * a.yr;
  b.xr = 0.25f * a.xr;
  b.xb = 0.25f * a.xb;
  b.P = 0.25f * a.P;
  b.gt = 0.25f * a.gt;
  b.gs = 0.25f * a.gs;
  b.gc = 0.25f * a.gc;
  dev_collide_pair<1>(m, a, usq3, ug, omt, omg, d[1], d[3], g[1], g[3]);
  dev_collide_pair<2>(m, a, usq3, ug, omt, omg, d[2], d[4], g[2], g[4]);
  dev_collide_pair<5>(m, b, usq3, ug, omt, omg, d[5], d[7], g[5], g[7]);
  dev_collide_pair<6>(m, b, usq3, ug, omt, omg, d[6], d[8], g[6], g[8]);
}

// ---- two directions per instruction (16-bit storage) ---------------------------
// The directions of one weight class pair up with their opposites as (1, 2) |
// (3, 4) and (5, 6) | (7, 8), so dev_collide_pair<1> and <2> (and <5> and <6>)
// are one computation on pairs.  dev_collide_x2 does them in the packed FP32x2
// arithmetic of sm_100-class GPUs (__ffma2_rn, __fadd2_rn, __fmul2_rn: one
// instruction for both directions, each result rounded as its scalar
// counterpart), halving the instructions of the eight moving directions; the
// 16-bit-storage kernels, bound by instruction issue, use it.
namespace x2 {
__device__ __forceinline__ float2 sp(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, sp(-1.0f), a); }

struct Class2 {
  float2 yr, xr, xb, P, gt, gs, gc;
};

// directions (I, I+1) and their opposites: dp = (d_I, d_I+1), dm = (d_opp I, d_opp I+1)
__device__ __forceinline__ void collide_set(const Class2& k, float2 t, float2 eg, float2 nusq3, float2 nug, float2 omt,
                                            float2 omg, float2& dp, float2& dm, float2& gp, float2& gm) {
  const float2 s2 = fma(t, t, nusq3);
  const float2 B = fma(eg, t, nug);
  const float2 Z = fma(k.xr, s2, fma(k.P, B, k.xb));
  const float2 V = fma(k.yr, t, mul(k.P, eg));
  dp = fma(omt, dp, add(Z, V));
  dm = fma(omt, dm, sub(Z, V));
  const float2 G = fma(k.gs, s2, k.gc);
  const float2 Gt = mul(k.gt, t);
  gp = fma(omg, gp, add(G, Gt));
  gm = fma(omg, gm, sub(G, Gt));
}
}  // namespace x2

__device__ __forceinline__ void dev_collide_x2(const DevCoef& c, const DevMacro& m, float (&d)[9], float (&g)[9]) {
  using namespace x2;
  const float base = fmaf(3.0f * m.psi, m.mu, m.drho);  // 3p - 1
  const float ug = m.ux * m.gx + m.uy * m.gy;
  const float usq3 = 3.0f * (m.ux * m.ux + m.uy * m.uy);
  float2 g12 = make_float2(g[1], g[2]), g34 = make_float2(g[3], g[4]);
  float2 g56 = make_float2(g[5], g[6]), g78 = make_float2(g[7], g[8]);
  const float2 Sp = add(add(g12, g34), add(g56, g78));
  const float S = Sp.x + Sp.y;
  const float itg = c.inv_tau_g;
  {  // rest direction, as dev_collide
    constexpr float w0 = wgt<0>();
    const float deq = fmaf(w0, m.drho, fmaf(-0.5f * w0 * m.rho, usq3, -c.c_a0 * m.psi * m.mu));
    const float F = -(3.0f * w0) * m.pref * ug;
    d[0] = fmaf(deq - d[0], m.inv_tau, d[0]) + F;
    const float dg = fmaf(-0.5f * w0 * m.psi, usq3, S - c.c_b0 * m.mu);
    g[0] = fmaf(dg, itg, g[0]);
  }
  Class2 a;  // w = 1/9
  const float yr = (1.0f / 9.0f) * m.inv_tau * m.rho;
  a.yr = sp(yr);
  a.xr = sp(0.5f * yr);
  a.xb = sp((1.0f / 9.0f) * m.inv_tau * base);
  a.P = sp((1.0f / 3.0f) * m.pref);
  const float gt = ((1.0f / 9.0f) * itg) * m.psi;
  a.gt = sp(gt);
  a.gs = sp(0.5f * gt);
  a.gc = sp(((1.0f / 9.0f) * itg) * c.three_gamma * m.mu);
  Class2 b;  // w = 1/36 = (1/9) / 4
  b.yr = mul(sp(0.25f), a.yr);
  b.xr = mul(sp(0.25f), a.xr);
  b.xb = mul(sp(0.25f), a.xb);
  b.P = mul(sp(0.25f), a.P);
  b.gt = mul(sp(0.25f), a.gt);
  b.gs = mul(sp(0.25f), a.gs);
  b.gc = mul(sp(0.25f), a.gc);
  const float2 omt = sp(1.0f - m.inv_tau), omg = sp(1.0f - itg);
  const float2 nusq3 = sp(-usq3), nug = sp(-ug);
  float2 d12 = make_float2(d[1], d[2]), d34 = make_float2(d[3], d[4]);
  float2 d56 = make_float2(d[5], d[6]), d78 = make_float2(d[7], d[8]);
  // e.u and e.grad psi of directions (1, 2): (u_x, u_y); of (5, 6): (u_x + u_y, u_y - u_x)
  const float2 u = make_float2(m.ux, m.uy), gr = make_float2(m.gx, m.gy);
  collide_set(a, mul(sp(3.0f), u), gr, nusq3, nug, omt, omg, d12, d34, g12, g34);
  const float2 u56 = make_float2(m.ux + m.uy, m.uy - m.ux), g56r = make_float2(m.gx + m.gy, m.gy - m.gx);
  collide_set(b, mul(sp(3.0f), u56), g56r, nusq3, nug, omt, omg, d56, d78, g56, g78);
  d[1] = d12.x; d[2] = d12.y; d[3] = d34.x; d[4] = d34.y;
  d[5] = d56.x; d[6] = d56.y; d[7] = d78.x; d[8] = d78.y;
  g[1] = g12.x; g[2] = g12.y; g[3] = g34.x; g[4] = g34.y;
  g[5] = g56.x; g[6] = g56.y; g[7] = g78.x; g[8] = g78.y;
}

// The collision of the staged kernels: packed pairs for 16-bit storage
template <typename SF>
__device__ __forceinline__ void dev_collide_for(const DevCoef& c, const DevMacro& m, float (&d)[9], float (&g)[9]) {
  if constexpr (!std::is_same_v<SF, float>) dev_collide_x2(c, m, d, g);
  else dev_collide(c, m, d, g);
}

// ---- Zou-He on deviations ----------------------------------------------------
__device__ __forceinline__ float dev_inlet_D(const float (&d)[9], float gx, float mu) {
  return ((d[0] + d[2]) + d[4]) + 2.0f * ((d[3] + d[6]) + d[7]) - 0.5f * gx * mu;
}

// rho_inlet - 1 of a row from its deviations (fingering.py:303-304)
__device__ __forceinline__ float dev_inlet_drho(const float (&d)[9], float ux, float gx, float mu) {
  return (dev_inlet_D(d, gx, mu) + ux) * __frcp_rn(1.0f - ux);
}

__device__ __forceinline__ void dev_zou_he_f(const DevCoef& c, int variant, int H, int W, int x, int y, float (&d)[9],
                                             float ux, float gx, float gy, float mu, float drho_nb) {
  const float gm6 = gx * mu * (1.0f / 6.0f), gm4 = 0.25f * gy * mu;
  if (x == 0) {
    if (variant == FD_VARIANT_WALLS && y == 0) {          // fingering.py:334-348
      d[1] = d[3];
      d[2] = d[4];
      d[5] = d[7];
      d[6] = 0.5f * (drho_nb - ((((d[0] + d[1]) + (d[2] + d[3])) + (d[4] + d[5])) + d[7]));
      d[8] = d[6];
    } else if (variant == FD_VARIANT_WALLS && y == H - 1) {  // fingering.py:350-364
      d[1] = d[3];
      d[4] = d[2];
      d[8] = d[6];
      d[5] = 0.5f * (drho_nb - ((((d[0] + d[1]) + (d[2] + d[3])) + (d[4] + d[6])) + d[8]));
      d[7] = d[5];
    } else {                                               // fingering_periodic.py:276-302
      const float rho_in = (1.0f + dev_inlet_D(d, gx, mu)) * __frcp_rn(1.0f - ux);
      const float a = ux * rho_in;
      d[1] = d[3] + (2.0f / 3.0f) * a - gm6;
      d[5] = d[7] - 0.5f * (d[2] - d[4]) + (1.0f / 6.0f) * a - gm6 - gm4;
      d[8] = d[6] + 0.5f * (d[2] - d[4]) + (1.0f / 6.0f) * a - gm6 + gm4;
    }
  }
  if (x == W - 1) {                                        // fingering_periodic.py:312-324
    const float D = ((d[0] + d[2]) + d[4]) + 2.0f * ((d[1] + d[5]) + d[8]) + 0.5f * gx * mu;
    // velocity outlet: a = u_x rho_out with rho_out = (1 + D) / (1 + u_x); pressure outlet
    // (FD_OUTLET_PRESSURE): rho_out = 1 and u_x = D, so a = D and the coefficient is 2/3
    const float a = c.p_out ? D : ux * ((1.0f + D) * __frcp_rn(1.0f + ux));
    d[3] = d[1] - (c.p_out ? (2.0f / 3.0f) : c.out_coef) * a + gm6;
    d[6] = d[8] - 0.5f * (d[2] - d[4]) - (1.0f / 6.0f) * a + gm4 + gm6;
    d[7] = d[5] + 0.5f * (d[2] - d[4]) - (1.0f / 6.0f) * a - gm4 + gm6;
    if (variant == FD_VARIANT_WALLS) {                     // fingering.py:387-390
      if (y == 0) d[2] = d[4];
      if (y == H - 1) d[4] = d[2];
    }
  }
}

__device__ __forceinline__ void dev_zou_he_g(const DevCoef& c, int variant, int H, int W, int x, int y, float (&g)[9]) {
  if (x == 0) {
    // 1 - g_0 (and -1 - g_0 at the outlet) first: g_0 is close to +1 (-1) there, so
    // the difference is exact and the small populations are not rounded against 1
    if (variant == FD_VARIANT_WALLS && y == 0) {
      g[1] = g[3];
      g[2] = g[4];
      g[5] = g[7];
      g[6] = 0.5f * ((1.0f - g[0]) - (((g[1] + g[2]) + (g[3] + g[4])) + (g[5] + g[7])));  // w6 / (w6 + w8)
      g[8] = g[6];
    } else if (variant == FD_VARIANT_WALLS && y == H - 1) {
      g[1] = g[3];
      g[4] = g[2];
      g[8] = g[6];
      g[5] = 0.5f * ((1.0f - g[0]) - (((g[1] + g[2]) + (g[3] + g[4])) + (g[6] + g[8])));
      g[7] = g[5];
    } else {
      const float psi_in = (1.0f - g[0]) - (((g[2] + g[3]) + (g[4] + g[6])) + g[7]);
      g[1] = (2.0f / 3.0f) * psi_in;   // w1 / (w1 + w5 + w8)
      g[5] = (1.0f / 6.0f) * psi_in;
      g[8] = (1.0f / 6.0f) * psi_in;
    }
  }
  if (x == W - 1) {
    const float psi_out = (-1.0f - g[0]) - (((g[1] + g[2]) + (g[4] + g[5])) + g[8]);
    g[3] = (2.0f / 3.0f) * psi_out;
    g[6] = (1.0f / 6.0f) * psi_out;
    g[7] = (1.0f / 6.0f) * psi_out;
    if (variant == FD_VARIANT_WALLS) {
      if (y == 0) g[2] = g[4];
      if (y == H - 1) g[4] = g[2];
    }
  }
}

}  // namespace fd
