// Per-cell physics of the two-phase free-energy D2Q9 LBM.
//
// Every expression keeps the operand order of the reference's numpy
// expressions (left-to-right, sequential sums over directions).  Translation
// units built with -fmad=false therefore reproduce the reference's FP64
// results bit for bit; units built with contraction enabled get the same
// formulas with FMAs.
#pragma once

#include "fd_common.cuh"

namespace fd {

// Macroscopic state of one fluid cell at the start of a collision.
template <typename T>
struct Macro {
  T rho, ux, uy, p, mu, tau_mix, psi, gx, gy;
};

// psi stencils (fingering_periodic.py:214-256): arguments are the 3x3
// neighbourhood after psi_wall / ghost substitution.
template <typename T>
__device__ __forceinline__ T grad_x(T E, T Wv, T NE, T NW, T SE, T SW) {
  return (((((T(4) * E + T(-4) * Wv) + NE) - NW) - SW) + SE) / T(12);
}
template <typename T>
__device__ __forceinline__ T grad_y(T N, T S, T NE, T NW, T SE, T SW) {
  return (((((T(4) * N + T(-4) * S) + NE) + NW) - SW) - SE) / T(12);
}
template <typename T>
__device__ __forceinline__ T laplacian(T C, T E, T Wv, T N, T S, T NE, T NW, T SE, T SW) {
  return ((((((((T(-20) * C + T(4) * N) + T(4) * E) + T(4) * Wv) + T(4) * S) + NE) + NW) + SW) + SE) / T(6);
}

// getMu / getMu_plain (fingering_periodic.py:141-149)
template <typename T>
__device__ __forceinline__ T chem_pot(const Coef<T>& c, T psi, T lap) {
  return ((c.a * psi) * (T(1) - psi * psi)) - c.kappa * lap;
}

// getMix_tau (fingering_periodic.py:201-208)
template <typename T>
__device__ __forceinline__ T mix_tau_of(const Coef<T>& c, T rho, T psi) {
  const T v1 = c.eta_n / rho;
  const T v2 = c.eta_n_M / rho;
  const T mv = ((T(2) * v1) * v2) / ((v1 * (T(1) - psi)) + (v2 * (T(1) + psi)));
  return T(3) * mv + T(0.5);
}

// getP (fingering_periodic.py:123-124)
template <typename T>
__device__ __forceinline__ T pressure_of(const Coef<T>& c, T rho, T psi, T mu) {
  return c.one_third * rho + psi * mu;
}

// np.sum over the nine directions (sequential, as numpy reduces axis 0)
template <typename T>
__device__ __forceinline__ T sum9(const T (&v)[9]) {
  T s = v[0];
#pragma unroll
  for (int i = 1; i < 9; ++i) s = s + v[i];
  return s;
}

// sum_i f_i e_ix and sum_i f_i e_iy in the order of fingering_periodic.py:128-129, 136-137
template <typename T>
__device__ __forceinline__ T mom_x(const T (&f)[9]) { return ((((f[1] - f[3]) + f[5]) - f[6]) - f[7]) + f[8]; }
template <typename T>
__device__ __forceinline__ T mom_y(const T (&f)[9]) { return ((((f[2] - f[4]) + f[5]) + f[6]) - f[7]) - f[8]; }

// getUx / getUy (fingering_periodic.py:126-139)
template <typename T>
__device__ __forceinline__ T velocity_of(T mom, T mu, T grad, T rho) {
  return (mom + ((mu * grad) / T(2))) / rho;
}

// the same with half the body force density rho b added (Guo forcing; the
// FD_VARIANT_PERIODIC_XY extension), or velocity_of when c.body == 0
template <typename T>
__device__ __forceinline__ T velocity_c(const Coef<T>& c, T mom, T mu, T grad, T rho, T b) {
  if (!c.body) return velocity_of(mom, mu, grad, rho);
  return ((mom + ((mu * grad) / T(2))) + ((rho * b) / T(2))) / rho;
}

// Macroscopic fields of one fluid cell from its populations, psi and the
// psi stencils, in the order of fingering_periodic.py:470-479.
template <typename T>
__device__ __forceinline__ Macro<T> macros_of(const Coef<T>& c, const T (&f)[9], T psi, T gx, T gy, T lap) {
  Macro<T> m;
  m.rho = sum9(f);
  m.psi = psi;
  m.gx = gx;
  m.gy = gy;
  m.mu = chem_pot(c, psi, lap);
  m.ux = velocity_c(c, mom_x(f), m.mu, gx, m.rho, c.bx);
  m.uy = velocity_c(c, mom_y(f), m.mu, gy, m.rho, c.by);
  m.p = pressure_of(c, m.rho, psi, m.mu);
  m.tau_mix = mix_tau_of(c, m.rho, psi);
  return m;
}

// Equilibria and forcing of direction i (fingering_periodic.py:155-199).
template <typename T>
struct CollisionTerms {
  T usq, inv_t, pref, A0, A18, B0, B18;
};

template <typename T>
__device__ __forceinline__ CollisionTerms<T> collision_terms(const Coef<T>& c, const Macro<T>& m) {
  CollisionTerms<T> t;
  t.usq = m.ux * m.ux + m.uy * m.uy;
  t.inv_t = T(1) / m.tau_mix;
  t.pref = T(1) - T(1) / (T(2) * m.tau_mix);
  t.A0 = (m.rho - c.c_a0 * m.p) / c.w[0];
  t.A18 = T(3) * m.p;
  t.B0 = (m.psi - c.c_b0 * m.mu) / c.w[0];
  t.B18 = c.c_b18 * m.mu;
  return t;
}

template <int I, typename T>
__device__ __forceinline__ void dir_terms(const Coef<T>& c, const Macro<T>& m, const CollisionTerms<T>& t,
                                          T& feq, T& geq, T& F) {
  constexpr T ex = T(ex_of(I)), ey = T(ey_of(I));
  const T eu = ex * m.ux + ey * m.uy;
  const T q = (T(3) * eu + T(4.5) * (eu * eu)) - T(1.5) * t.usq;
  feq = c.w[I] * ((I == 0 ? t.A0 : t.A18) + m.rho * q);
  geq = c.w[I] * ((I == 0 ? t.B0 : t.B18) + m.psi * q);
  const T Ax = ((ex - m.ux) * T(3)) + ((ex * eu) * T(9));
  const T Ay = ((ey - m.uy) * T(3)) + ((ey * eu) * T(9));
  F = ((m.mu * c.w[I]) * t.pref) * (Ax * m.gx + Ay * m.gy);
  if (c.body) F = F + ((m.rho * c.w[I]) * t.pref) * (Ax * c.bx + Ay * c.by);  // body force density rho b
}

template <int I, typename T>
__device__ __forceinline__ void collide_dir(const Coef<T>& c, const Macro<T>& m, const CollisionTerms<T>& t,
                                            T& f, T& g) {
  T feq, geq, F;
  dir_terms<I>(c, m, t, feq, geq, F);
  f = (f - t.inv_t * (f - feq)) + F;       // getF (fingering_periodic.py:258-260)
  g = g - c.tau_inv * (g - geq);           // getG (fingering_periodic.py:262-264)
}

template <typename T>
__device__ __forceinline__ void collide(const Coef<T>& c, const Macro<T>& m, T (&f)[9], T (&g)[9]) {
  const CollisionTerms<T> t = collision_terms(c, m);
  collide_dir<0>(c, m, t, f[0], g[0]);
  collide_dir<1>(c, m, t, f[1], g[1]);
  collide_dir<2>(c, m, t, f[2], g[2]);
  collide_dir<3>(c, m, t, f[3], g[3]);
  collide_dir<4>(c, m, t, f[4], g[4]);
  collide_dir<5>(c, m, t, f[5], g[5]);
  collide_dir<6>(c, m, t, f[6], g[6]);
  collide_dir<7>(c, m, t, f[7], g[7]);
  collide_dir<8>(c, m, t, f[8], g[8]);
}

// ---------------------------------------------------------------------------
// Zou-He rules on one cell's post-stream populations
// ---------------------------------------------------------------------------
// rho_inlet (fingering_periodic.py:276-277)
template <typename T>
__device__ __forceinline__ T inlet_rho(const T (&f)[9], T ux, T gx, T mu) {
  return (T(1) / (T(1) - ux)) * ((((f[0] + f[2]) + f[4]) + T(2) * ((f[3] + f[6]) + f[7])) - ((gx * mu) / T(2)));
}

// fingering_periodic.py:281-302 (and fingering.py:308-332 on rows 1..H-2)
template <typename T>
__device__ __forceinline__ void inlet_f(const Coef<T>& c, T (&f)[9], T ux, T gx, T gy, T mu) {
  const T r = inlet_rho(f, ux, gx, mu);
  f[1] = (f[3] + (c.two_thirds * ux) * r) - ((gx * mu) / T(6));
  f[5] = (((f[7] - T(0.5) * (f[2] - f[4])) + (c.one_sixth * ux) * r) - ((gx * mu) / T(6))) - ((gy * mu) / T(4));
  f[8] = (((f[6] + T(0.5) * (f[2] - f[4])) + (c.one_sixth * ux) * r) - ((gx * mu) / T(6))) + ((gy * mu) / T(4));
}

template <typename T>
__device__ __forceinline__ void inlet_g(const Coef<T>& c, T (&g)[9]) {
  const T psi_in = T(1) - (((((g[0] + g[2]) + g[3]) + g[4]) + g[6]) + g[7]);
  g[1] = (c.w[1] * psi_in) / c.wsum_in;
  g[5] = (c.w[5] * psi_in) / c.wsum_in;
  g[8] = (c.w[8] * psi_in) / c.wsum_in;
}

// bottom-left inlet corner (fingering.py:334-348); rho1 = rho_inlet of row 1
template <typename T>
__device__ __forceinline__ void inlet_corner_bottom_f(T (&f)[9], T rho1) {
  f[1] = f[3];
  f[2] = f[4];
  f[5] = f[7];
  f[6] = T(0.5) * (rho1 - ((((((f[0] + f[1]) + f[2]) + f[3]) + f[4]) + f[5]) + f[7]));
  f[8] = f[6];
}
template <typename T>
__device__ __forceinline__ void inlet_corner_bottom_g(const Coef<T>& c, T (&g)[9]) {
  g[1] = g[3];
  g[2] = g[4];
  g[5] = g[7];
  g[6] = (c.w[6] * (T(1) - ((((((g[0] + g[1]) + g[2]) + g[3]) + g[4]) + g[5]) + g[7]))) / c.wsum_68;
  g[8] = g[6];
}
// top-left inlet corner (fingering.py:350-364); rhoH2 = rho_inlet of row H-2
template <typename T>
__device__ __forceinline__ void inlet_corner_top_f(T (&f)[9], T rhoH2) {
  f[1] = f[3];
  f[4] = f[2];
  f[8] = f[6];
  f[5] = T(0.5) * (rhoH2 - ((((((f[0] + f[1]) + f[2]) + f[3]) + f[4]) + f[6]) + f[8]));
  f[7] = f[5];
}
template <typename T>
__device__ __forceinline__ void inlet_corner_top_g(const Coef<T>& c, T (&g)[9]) {
  g[1] = g[3];
  g[4] = g[2];
  g[8] = g[6];
  g[5] = (c.w[5] * (T(1) - ((((((g[0] + g[1]) + g[2]) + g[3]) + g[4]) + g[6]) + g[8]))) / c.wsum_57;
  g[7] = g[5];
}

// fingering_periodic.py:305-324 / fingering.py:369-385.  With FD_OUTLET_PRESSURE
// (an extension) rho_out = 1 is imposed instead and u_x = S / rho_out - 1
// follows from the same known-population sum S; the coefficient of f3 is then
// the standard 2/3, so that the outlet cell's density is exactly rho_out.
template <typename T>
__device__ __forceinline__ void outlet_f(const Coef<T>& c, T (&f)[9], T ux, T gx, T gy, T mu) {
  const T S = (((f[0] + f[2]) + f[4]) + T(2) * ((f[1] + f[5]) + f[8])) + ((gx * mu) / T(2));
  T r, coef;
  if (c.p_out) {
    r = T(1);
    ux = S - T(1);
    coef = c.two_thirds;
  } else {
    r = (T(1) / (T(1) + ux)) * S;
    coef = c.out_coef;
  }
  f[3] = (f[1] - (coef * ux) * r) + ((gx * mu) / T(6));
  f[6] = (((f[8] - T(0.5) * (f[2] - f[4])) - (c.one_sixth * ux) * r) + ((gy * mu) / T(4))) + ((gx * mu) / T(6));
  f[7] = (((f[5] + T(0.5) * (f[2] - f[4])) - (c.one_sixth * ux) * r) - ((gy * mu) / T(4))) + ((gx * mu) / T(6));
}
template <typename T>
__device__ __forceinline__ void outlet_g(const Coef<T>& c, T (&g)[9]) {
  const T psi_out = T(-1) - (((((g[0] + g[1]) + g[2]) + g[4]) + g[5]) + g[8]);
  g[3] = (c.w[3] * psi_out) / c.wsum_out;
  g[6] = (c.w[6] * psi_out) / c.wsum_out;
  g[7] = (c.w[7] * psi_out) / c.wsum_out;
}

}  // namespace fd
