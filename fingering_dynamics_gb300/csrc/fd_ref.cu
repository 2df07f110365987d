// Reference-order kernels: one kernel per function of the reference's step
// (fingering_periodic.py / fingering.py / bounce_back.py), one thread per
// cell.  Built with -fmad=false so that, in FP64, each kernel reproduces the
// reference's numpy arithmetic bit for bit.  These are the drop-in entry
// points for callers that drive the reference's loop body phase by phase;
// the fused kernel (fd_fused_*.cu) is the fast path.
#include <cstddef>

#include "fd_host.h"
#include "fd_zouhe.cuh"

namespace fd {
namespace {

constexpr int kBlock = 256;

template <typename T>
struct Fields {
  T *f, *g, *psi, *npx, *npy, *np2, *rho, *ux, *uy, *p, *mu, *mix_tau;
};

template <typename T>
Fields<T> typed(const fd_fields& a) {
  return Fields<T>{(T*)a.f,   (T*)a.g,  (T*)a.psi, (T*)a.npx, (T*)a.npy, (T*)a.np2,
                   (T*)a.rho, (T*)a.ux, (T*)a.uy,  (T*)a.p,   (T*)a.mu,  (T*)a.mix_tau};
}

struct Shape {
  int H, W, variant;
  size_t P;  // plane size H*W
};

inline Shape shape_of(const fd_params& p) { return Shape{p.H, p.W, p.variant, (size_t)p.H * (size_t)p.W}; }

inline dim3 grid_cells(const Shape& s) { return dim3((unsigned)((s.P + kBlock - 1) / kBlock)); }

// psi of (x, y) as the reference's stencils see it: psi_wall on solid cells
// (fingering_periodic.py:216-217), +1 / -1 ghost columns left / right
// (fingering_periodic.py:94-95), y wrapped (fingering_periodic.py, np.roll)
// or psi_wall ghost rows including their corners (fingering.py:102,224).
// FD_VARIANT_PERIODIC_XY wraps x as well.
template <typename T>
__device__ __forceinline__ T psi_nb(const T* __restrict__ psi, const uint16_t* __restrict__ mask, const Shape& s,
                                    T psi_wall, int x, int y) {
  if (y < 0 || y >= s.H) {
    if (s.variant == FD_VARIANT_WALLS) return psi_wall;
    y = wrap(y, s.H);
  }
  if (s.variant == FD_VARIANT_PERIODIC_XY) {
    x = wrap(x, s.W);
  } else {
    if (x < 0) return T(1);
    if (x >= s.W) return T(-1);
  }
  const size_t q = (size_t)y * s.W + x;
  return (mask[q] & SOLID) ? psi_wall : psi[q];
}

template <typename T>
__device__ __forceinline__ void stencil_at(const T* __restrict__ psi, const uint16_t* __restrict__ mask,
                                           const Shape& s, T psi_wall, int x, int y, T& gx, T& gy, T& lap) {
  const T C = psi_nb(psi, mask, s, psi_wall, x, y);
  const T E = psi_nb(psi, mask, s, psi_wall, x + 1, y), Wv = psi_nb(psi, mask, s, psi_wall, x - 1, y);
  const T N = psi_nb(psi, mask, s, psi_wall, x, y + 1), S = psi_nb(psi, mask, s, psi_wall, x, y - 1);
  const T NE = psi_nb(psi, mask, s, psi_wall, x + 1, y + 1), NW = psi_nb(psi, mask, s, psi_wall, x - 1, y + 1);
  const T SE = psi_nb(psi, mask, s, psi_wall, x + 1, y - 1), SW = psi_nb(psi, mask, s, psi_wall, x - 1, y - 1);
  gx = grad_x(E, Wv, NE, NW, SE, SW);
  gy = grad_y(N, S, NE, NW, SE, SW);
  lap = laplacian(C, E, Wv, N, S, NE, NW, SE, SW);
}

template <typename T>
__device__ __forceinline__ Macro<T> load_macro(const Fields<T>& F, size_t q) {
  Macro<T> m;
  m.rho = F.rho[q]; m.ux = F.ux[q]; m.uy = F.uy[q]; m.p = F.p[q]; m.mu = F.mu[q];
  m.tau_mix = F.mix_tau[q]; m.psi = F.psi[q]; m.gx = F.npx[q]; m.gy = F.npy[q];
  return m;
}

// --- Compute.__init__ ------------------------------------------------------
template <typename T>
__global__ void k_init_psi(Shape s, T psi_wall, const uint16_t* __restrict__ mask, const double* __restrict__ psi0,
                           const double* __restrict__ rho0, Fields<T> F) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P) return;
  const bool solid = mask[q] & SOLID;
  F.psi[q] = solid ? psi_wall : (T)psi0[q];                  // fingering_periodic.py:90-93
  F.rho[q] = rho0 ? (T)rho0[q] : T(1);                       // fingering_periodic.py:103
}

template <typename T>
__global__ void k_init_rest(Shape s, Coef<T> c, unsigned flags, const uint16_t* __restrict__ mask, Fields<T> F) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P) return;
  const int x = (int)(q % s.W), y = (int)(q / s.W);
  T gx, gy, lap;
  stencil_at(F.psi, mask, s, c.psi_wall, x, y, gx, gy, lap);
  F.npx[q] = gx; F.npy[q] = gy; F.np2[q] = lap;
  if (mask[q] & SOLID) {
#pragma unroll
    for (int i = 0; i < 9; ++i) { F.f[i * s.P + q] = T(0); F.g[i * s.P + q] = T(0); }
    F.ux[q] = T(0); F.uy[q] = T(0); F.p[q] = T(0); F.mu[q] = T(0); F.mix_tau[q] = T(0);
    return;
  }
  Macro<T> m;
  m.rho = F.rho[q];
  m.psi = F.psi[q];
  m.gx = gx; m.gy = gy;
  m.p = pressure_of(c, m.rho, m.psi, T(0));                  // getP with mu = 0 (fingering_periodic.py:111,117)
  m.mu = (flags & FD_INIT_MU) ? chem_pot(c, m.psi, lap) : T(0);               // fingering.py:122
  if (flags & FD_INIT_VELOCITY) {  // caller-supplied u (no reference counterpart: the scripts start at rest)
    m.ux = F.ux[q];
    m.uy = F.uy[q];
  } else {
    m.ux = T(0);
    m.uy = (flags & FD_INIT_UY) ? velocity_of(T(0), m.mu, gy, m.rho) : T(0);  // fingering.py:123
  }
  m.tau_mix = mix_tau_of(c, m.rho, m.psi);
  F.ux[q] = m.ux; F.uy[q] = m.uy; F.p[q] = m.p; F.mu[q] = m.mu; F.mix_tau[q] = m.tau_mix;
  const CollisionTerms<T> t = collision_terms(c, m);
  T feq[9], geq[9], Fi;
  dir_terms<0>(c, m, t, feq[0], geq[0], Fi); dir_terms<1>(c, m, t, feq[1], geq[1], Fi);
  dir_terms<2>(c, m, t, feq[2], geq[2], Fi); dir_terms<3>(c, m, t, feq[3], geq[3], Fi);
  dir_terms<4>(c, m, t, feq[4], geq[4], Fi); dir_terms<5>(c, m, t, feq[5], geq[5], Fi);
  dir_terms<6>(c, m, t, feq[6], geq[6], Fi); dir_terms<7>(c, m, t, feq[7], geq[7], Fi);
  dir_terms<8>(c, m, t, feq[8], geq[8], Fi);
#pragma unroll
  for (int i = 0; i < 9; ++i) { F.f[i * s.P + q] = feq[i]; F.g[i * s.P + q] = geq[i]; }
}

// --- first-order non-equilibrium part of a restart (no reference counterpart) ---
// A state rebuilt from fields (fd_compute_init with FD_INIT_VELOCITY) is the
// equilibrium of those fields; a flow with velocity gradients also carries the
// first-order Chapman-Enskog part of its populations.  This kernel adds it:
//   f_i += -3 w_i tau_mix Q_i : S(rho u),   g_i += -3 w_i tau Q_i : S(psi u)
// with Q_i = e_i e_i - I/3 and S(v) the symmetric part of grad v from central
// differences over fluid neighbours (one-sided next to solid cells or the x
// edges, zero where neither neighbour is fluid).  sum_i w_i Q_i = 0 and
// sum_i w_i Q_i e_i = 0, so density, psi and momentum are unchanged.  Fluid
// cells only; fields must hold rho, psi, ux, uy, mix_tau of the state.
template <typename T>
__global__ void k_nonequilibrium(Shape s, Coef<T> c, const uint16_t* __restrict__ mask, Fields<T> F) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P || (mask[q] & SOLID)) return;
  const int x = (int)(q % s.W), y = (int)(q / s.W);
  // (rho u, psi u) at a neighbour, false if it is solid or outside the lattice
  auto flux = [&](int xx, int yy, T (&v)[4]) -> bool {
    if (yy < 0 || yy >= s.H) {
      if (s.variant == FD_VARIANT_WALLS) return false;
      yy = wrap(yy, s.H);
    }
    if (xx < 0 || xx >= s.W) {
      if (s.variant != FD_VARIANT_PERIODIC_XY) return false;
      xx = wrap(xx, s.W);
    }
    const size_t k = (size_t)yy * s.W + xx;
    if (mask[k] & SOLID) return false;
    v[0] = F.rho[k] * F.ux[k];
    v[1] = F.rho[k] * F.uy[k];
    v[2] = F.psi[k] * F.ux[k];
    v[3] = F.psi[k] * F.uy[k];
    return true;
  };
  T vc[4], vp[4], vm[4], dx[4], dy[4];
  flux(x, y, vc);
  const bool xp = flux(x + 1, y, vp), xm = flux(x - 1, y, vm);
#pragma unroll
  for (int k = 0; k < 4; ++k)
    dx[k] = (xp && xm) ? T(0.5) * (vp[k] - vm[k]) : xp ? vp[k] - vc[k] : xm ? vc[k] - vm[k] : T(0);
  const bool yp = flux(x, y + 1, vp), ym = flux(x, y - 1, vm);
#pragma unroll
  for (int k = 0; k < 4; ++k)
    dy[k] = (yp && ym) ? T(0.5) * (vp[k] - vm[k]) : yp ? vp[k] - vc[k] : ym ? vc[k] - vm[k] : T(0);
  // S of rho u (index 0/1) and of psi u (2/3)
  const T fxx = dx[0], fyy = dy[1], fxy = T(0.5) * (dy[0] + dx[1]);
  const T gxx = dx[2], gyy = dy[3], gxy = T(0.5) * (dy[2] + dx[3]);
  const T tf = F.mix_tau[q], tg = T(1) / c.tau_inv;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const T ex = (T)ex_of(i), ey = (T)ey_of(i);
    const T qxx = ex * ex - T(1) / T(3), qyy = ey * ey - T(1) / T(3), qxy = ex * ey;
    const T qsf = qxx * fxx + qyy * fyy + T(2) * qxy * fxy;
    const T qsg = qxx * gxx + qyy * gyy + T(2) * qxy * gxy;
    F.f[i * s.P + q] += T(-3) * c.w[i] * tf * qsf;
    F.g[i * s.P + q] += T(-3) * c.w[i] * tg * qsg;
  }
}

// --- collision (fingering_periodic.py:455-460) -----------------------------
template <typename T>
__global__ void k_collide(Shape s, Coef<T> c, const uint16_t* __restrict__ mask, Fields<T> F) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P || (mask[q] & SOLID)) return;
  const Macro<T> m = load_macro(F, q);
  T f[9], g[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) { f[i] = F.f[i * s.P + q]; g[i] = F.g[i * s.P + q]; }
  collide(c, m, f, g);
#pragma unroll
  for (int i = 0; i < 9; ++i) { F.f[i * s.P + q] = f[i]; F.g[i * s.P + q] = g[i]; }
}

template <int I, typename T>
__device__ __forceinline__ T term_of(const Coef<T>& c, const Macro<T>& m, const CollisionTerms<T>& t, int term,
                                     T f, T g) {
  T feq, geq, Fi;
  dir_terms<I>(c, m, t, feq, geq, Fi);
  switch (term) {
    case FD_TERM_LARGE_F: return Fi;
    case FD_TERM_FEQ: return feq;
    case FD_TERM_GEQ: return geq;
    case FD_TERM_F: return (f - t.inv_t * (f - feq)) + Fi;
    default: return g - c.tau_inv * (g - geq);
  }
}

template <typename T>
__global__ void k_collision_term(Shape s, Coef<T> c, int term, int j, const uint16_t* __restrict__ mask, Fields<T> F,
                                 T* __restrict__ out) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P || (mask[q] & SOLID)) return;
  const Macro<T> m = load_macro(F, q);
  const CollisionTerms<T> t = collision_terms(c, m);
  const T f = F.f[j * s.P + q], g = F.g[j * s.P + q];
  T r;
  switch (j) {
    case 0: r = term_of<0>(c, m, t, term, f, g); break;
    case 1: r = term_of<1>(c, m, t, term, f, g); break;
    case 2: r = term_of<2>(c, m, t, term, f, g); break;
    case 3: r = term_of<3>(c, m, t, term, f, g); break;
    case 4: r = term_of<4>(c, m, t, term, f, g); break;
    case 5: r = term_of<5>(c, m, t, term, f, g); break;
    case 6: r = term_of<6>(c, m, t, term, f, g); break;
    case 7: r = term_of<7>(c, m, t, term, f, g); break;
    default: r = term_of<8>(c, m, t, term, f, g); break;
  }
  out[q] = r;
}

// --- stream (fingering_periodic.py:327-343) --------------------------------
template <typename T>
__global__ void k_stream(Shape s, const T* __restrict__ sf, const T* __restrict__ sg, T* __restrict__ df,
                         T* __restrict__ dg) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P) return;
  const int x = (int)(q % s.W), y = (int)(q / s.W);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const size_t src = (size_t)wrap(y - ey_of(i), s.H) * s.W + wrap(x - ex_of(i), s.W);
    df[i * s.P + q] = sf[i * s.P + src];
    dg[i * s.P + q] = sg[i * s.P + src];
  }
}

// --- bounce-back as link bits (bounce_back.py:25-167, fingering.py:432-451) --
template <typename T>
__global__ void k_bounce_back(Shape s, const uint16_t* __restrict__ mask, const T* __restrict__ fb,
                              const T* __restrict__ gb, T* __restrict__ f, T* __restrict__ g) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P) return;
  const unsigned bits = mask[q] & 0xFFu;
  if (!bits) return;
#pragma unroll
  for (int i = 1; i < 9; ++i) {
    if (bits & (1u << (i - 1))) {
      f[i * s.P + q] = fb[opp_of(i) * s.P + q];
      g[i * s.P + q] = gb[opp_of(i) * s.P + q];
    }
  }
}

template <typename T>
__global__ void k_bottom_top_wall(int rows, int cols, ptrdiff_t ps, ptrdiff_t rs, const T* __restrict__ fb,
                                  const T* __restrict__ gb, T* __restrict__ f, T* __restrict__ g) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= cols) return;
  const ptrdiff_t top = (ptrdiff_t)(rows - 1) * rs + x;
  // fingering.py:435-451 in order; rows 0 and rows-1 coincide when rows == 1
  f[2 * ps + x] = fb[4 * ps + x]; g[2 * ps + x] = gb[4 * ps + x];
  f[4 * ps + top] = fb[2 * ps + top]; g[4 * ps + top] = gb[2 * ps + top];
  f[5 * ps + x] = fb[7 * ps + x]; g[5 * ps + x] = gb[7 * ps + x];
  f[6 * ps + x] = fb[8 * ps + x]; g[6 * ps + x] = gb[8 * ps + x];
  f[7 * ps + top] = fb[5 * ps + top]; g[7 * ps + top] = gb[5 * ps + top];
  f[8 * ps + top] = fb[6 * ps + top]; g[8 * ps + top] = gb[6 * ps + top];
}

// --- Zou-He ----------------------------------------------------------------
template <typename T>
__global__ void k_boundary_fields(Shape s, Coef<T> c, const uint16_t* __restrict__ mask, const T* __restrict__ psi,
                                  const T* __restrict__ np2, T* __restrict__ side) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * s.H) return;
  const int y = t % s.H, col = t / s.H, x = col ? s.W - 1 : 0;
  T gx, gy, lap;
  stencil_at(psi, mask, s, c.psi_wall, x, y, gx, gy, lap);
  const size_t q = (size_t)y * s.W + x;
  side[(3 * col + 0) * s.H + y] = gx;
  side[(3 * col + 1) * s.H + y] = gy;
  // getMu_plain reads the stored psi and nabla_psi2 (fingering_periodic.py:146-149)
  side[(3 * col + 2) * s.H + y] = chem_pot(c, psi[q], np2[q]);
}

template <typename T>
__device__ __forceinline__ void load_cell(const T* __restrict__ a, size_t P, size_t q, T (&v)[9]) {
#pragma unroll
  for (int i = 0; i < 9; ++i) v[i] = a[i * P + q];
}
template <typename T>
__device__ __forceinline__ void store_cell(T* __restrict__ a, size_t P, size_t q, const T (&v)[9]) {
#pragma unroll
  for (int i = 0; i < 9; ++i) a[i * P + q] = v[i];
}

template <typename T>
__global__ void k_zou_he(Shape s, Coef<T> c, int col, T* __restrict__ f, T* __restrict__ g, const T* __restrict__ side,
                         const double* __restrict__ inlet_ux) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= s.H) return;
  const int x = col ? s.W - 1 : 0;
  const size_t q = (size_t)y * s.W + x;
  T fv[9], gv[9];
  load_cell(f, s.P, q, fv);
  load_cell(g, s.P, q, gv);
  const T ux = (T)inlet_ux[y];
  T rho_nb = T(0);
  if (!col && s.variant == FD_VARIANT_WALLS && (y == 0 || y == s.H - 1)) {
    // rho_inlet of row 1 / H-2 (fingering.py:303-304 evaluates it on every row
    // before any row is modified; the populations it reads are not modified)
    const int yn = y == 0 ? 1 : s.H - 2;
    T fn[9];
    load_cell(f, s.P, (size_t)yn * s.W, fn);
    rho_nb = inlet_rho(fn, (T)inlet_ux[yn], side[0 * s.H + yn], side[2 * s.H + yn]);
  }
  const int o = col ? 3 : 0;
  zou_he_f(c, s.variant, s.H, s.W, x, y, fv, ux, side[(o + 0) * s.H + y], side[(o + 1) * s.H + y],
           side[(o + 2) * s.H + y], rho_nb);
  zou_he_g(c, s.variant, s.H, s.W, x, y, gv);
  store_cell(f, s.P, q, fv);
  store_cell(g, s.P, q, gv);
}

// --- macroscopic update (fingering_periodic.py:470-479) --------------------
template <typename T>
__global__ void k_rho_psi(Shape s, T psi_wall, const uint16_t* __restrict__ mask, Fields<T> F) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P) return;
  if (mask[q] & SOLID) { F.psi[q] = psi_wall; return; }
  T v[9];
  load_cell(F.f, s.P, q, v);
  F.rho[q] = sum9(v);
  load_cell(F.g, s.P, q, v);
  F.psi[q] = sum9(v);
}

template <typename T>
__global__ void k_macros(Shape s, Coef<T> c, const uint16_t* __restrict__ mask, Fields<T> F) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P) return;
  const int x = (int)(q % s.W), y = (int)(q / s.W);
  T gx, gy, lap;
  stencil_at(F.psi, mask, s, c.psi_wall, x, y, gx, gy, lap);
  F.npx[q] = gx; F.npy[q] = gy; F.np2[q] = lap;
  if (mask[q] & SOLID) return;
  T v[9];
  load_cell(F.f, s.P, q, v);
  const T rho = F.rho[q], psi = F.psi[q];
  const T mu = chem_pot(c, psi, lap);
  F.mu[q] = mu;
  F.ux[q] = velocity_c(c, mom_x(v), mu, gx, rho, c.bx);
  F.uy[q] = velocity_c(c, mom_y(v), mu, gy, rho, c.by);
  F.p[q] = pressure_of(c, rho, psi, mu);
  F.mix_tau[q] = mix_tau_of(c, rho, psi);
}

template <typename T>
__global__ void k_field(Shape s, Coef<T> c, int which, const uint16_t* __restrict__ mask, Fields<T> F,
                        T* __restrict__ out) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.P) return;
  const int x = (int)(q % s.W), y = (int)(q / s.W);
  const bool solid = mask[q] & SOLID;
  T gx, gy, lap, v[9];
  switch (which) {
    case FD_FIELD_NPX: stencil_at(F.psi, mask, s, c.psi_wall, x, y, gx, gy, lap); out[q] = gx; return;
    case FD_FIELD_NPY: stencil_at(F.psi, mask, s, c.psi_wall, x, y, gx, gy, lap); out[q] = gy; return;
    case FD_FIELD_NP2: stencil_at(F.psi, mask, s, c.psi_wall, x, y, gx, gy, lap); out[q] = lap; return;
    case FD_FIELD_MU_PLAIN: out[q] = chem_pot(c, F.psi[q], F.np2[q]); return;
    case FD_FIELD_PSI:
      if (solid) {
        out[q] = c.psi_wall;
      } else {
        load_cell(F.g, s.P, q, v);
        out[q] = sum9(v);
      }
      return;
    default: break;
  }
  if (solid) return;
  switch (which) {
    case FD_FIELD_RHO: load_cell(F.f, s.P, q, v); out[q] = sum9(v); return;
    case FD_FIELD_MU: out[q] = chem_pot(c, F.psi[q], F.np2[q]); return;
    case FD_FIELD_UX:
      load_cell(F.f, s.P, q, v);
      out[q] = velocity_c(c, mom_x(v), F.mu[q], F.npx[q], F.rho[q], c.bx);
      return;
    case FD_FIELD_UY:
      load_cell(F.f, s.P, q, v);
      out[q] = velocity_c(c, mom_y(v), F.mu[q], F.npy[q], F.rho[q], c.by);
      return;
    case FD_FIELD_P: out[q] = pressure_of(c, F.rho[q], F.psi[q], F.mu[q]); return;
    case FD_FIELD_MIX_TAU: out[q] = mix_tau_of(c, F.rho[q], F.psi[q]); return;
    default: return;
  }
}

// ---------------------------------------------------------------------------
// typed launchers
// ---------------------------------------------------------------------------
template <typename T>
int launch_init(const fd_params& p, const uint16_t* mask, const double* psi0, const double* rho0,
                const fd_fields& out, cudaStream_t st) {
  const Shape s = shape_of(p);
  const Coef<T> c = make_coef<T>(p);
  const Fields<T> F = typed<T>(out);
  k_init_psi<T><<<grid_cells(s), kBlock, 0, st>>>(s, c.psi_wall, mask, psi0, rho0, F);
  k_init_rest<T><<<grid_cells(s), kBlock, 0, st>>>(s, c, p.flags, mask, F);
  return check_launch("fd_compute_init");
}

template <typename T>
int launch_nonequilibrium(const fd_params& p, const uint16_t* mask, const fd_fields& fl, cudaStream_t st) {
  const Shape s = shape_of(p);
  k_nonequilibrium<T><<<grid_cells(s), kBlock, 0, st>>>(s, make_coef<T>(p), mask, typed<T>(fl));
  return check_launch("fd_add_nonequilibrium");
}

template <typename T>
int launch_collide(const fd_params& p, const uint16_t* mask, const fd_fields& fl, cudaStream_t st) {
  const Shape s = shape_of(p);
  k_collide<T><<<grid_cells(s), kBlock, 0, st>>>(s, make_coef<T>(p), mask, typed<T>(fl));
  return check_launch("fd_collide");
}

template <typename T>
int launch_term(const fd_params& p, int term, int j, const uint16_t* mask, const fd_fields& fl, void* out,
                cudaStream_t st) {
  const Shape s = shape_of(p);
  k_collision_term<T><<<grid_cells(s), kBlock, 0, st>>>(s, make_coef<T>(p), term, j, mask, typed<T>(fl), (T*)out);
  return check_launch("fd_collision_term");
}

template <typename T>
int launch_stream(const fd_params& p, const void* sf, const void* sg, void* df, void* dg, cudaStream_t st) {
  const Shape s = shape_of(p);
  k_stream<T><<<grid_cells(s), kBlock, 0, st>>>(s, (const T*)sf, (const T*)sg, (T*)df, (T*)dg);
  return check_launch("fd_stream");
}

template <typename T>
int launch_bb(const fd_params& p, const uint16_t* mask, const void* fb, const void* gb, void* f, void* g,
              cudaStream_t st) {
  const Shape s = shape_of(p);
  k_bounce_back<T><<<grid_cells(s), kBlock, 0, st>>>(s, mask, (const T*)fb, (const T*)gb, (T*)f, (T*)g);
  return check_launch("fd_bounce_back");
}

template <typename T>
int launch_btw(int rows, int cols, ptrdiff_t ps, ptrdiff_t rs, const void* fb, const void* gb, void* f, void* g,
               cudaStream_t st) {
  k_bottom_top_wall<T><<<(cols + kBlock - 1) / kBlock, kBlock, 0, st>>>(rows, cols, ps, rs, (const T*)fb,
                                                                         (const T*)gb, (T*)f, (T*)g);
  return check_launch("fd_bottom_top_wall");
}

template <typename T>
int launch_bfields(const fd_params& p, const uint16_t* mask, const void* psi, const void* np2, void* side,
                   cudaStream_t st) {
  const Shape s = shape_of(p);
  k_boundary_fields<T><<<(2 * s.H + kBlock - 1) / kBlock, kBlock, 0, st>>>(s, make_coef<T>(p), mask, (const T*)psi,
                                                                             (const T*)np2, (T*)side);
  return check_launch("fd_boundary_fields");
}

template <typename T>
int launch_zou_he(const fd_params& p, int col, void* f, void* g, const void* side, const double* ux, cudaStream_t st) {
  const Shape s = shape_of(p);
  k_zou_he<T><<<(s.H + kBlock - 1) / kBlock, kBlock, 0, st>>>(s, make_coef<T>(p), col, (T*)f, (T*)g,
                                                                (const T*)side, ux);
  return check_launch(col ? "fd_zou_he_outlet" : "fd_zou_he_inlet");
}

template <typename T>
int launch_rho_psi(const fd_params& p, const uint16_t* mask, const fd_fields& fl, cudaStream_t st) {
  const Shape s = shape_of(p);
  k_rho_psi<T><<<grid_cells(s), kBlock, 0, st>>>(s, (T)p.psi_wall, mask, typed<T>(fl));
  return check_launch("fd_update_rho_psi");
}

template <typename T>
int launch_macros(const fd_params& p, const uint16_t* mask, const fd_fields& fl, cudaStream_t st) {
  const Shape s = shape_of(p);
  k_macros<T><<<grid_cells(s), kBlock, 0, st>>>(s, make_coef<T>(p), mask, typed<T>(fl));
  return check_launch("fd_update_macros");
}

template <typename T>
int launch_field(const fd_params& p, int which, const uint16_t* mask, const fd_fields& fl, void* out,
                 cudaStream_t st) {
  const Shape s = shape_of(p);
  k_field<T><<<grid_cells(s), kBlock, 0, st>>>(s, make_coef<T>(p), which, mask, typed<T>(fl), (T*)out);
  return check_launch("fd_field");
}

int check_dtype(int dtype) {
  FD_REQUIRE(dtype == FD_F64 || dtype == FD_F32, FD_ERR_DTYPE,
             "the per-function entry points support FD_F64 and FD_F32 (got %d)", dtype);
  return FD_OK;
}

bool fields_ok(const fd_fields* a) {
  return a && a->f && a->g && a->psi && a->npx && a->npy && a->np2 && a->rho && a->ux && a->uy && a->p && a->mu &&
         a->mix_tau;
}

}  // namespace
}  // namespace fd

using namespace fd;

#define FD_DISPATCH(dtype, call) ((dtype) == FD_F64 ? call<double> : call<float>)

extern "C" {

int fd_compute_init(const fd_params* prm, int dtype, const uint16_t* mask, const double* psi0, const double* rho0,
                    const fd_fields* out, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(mask && psi0 && fields_ok(out), FD_ERR_ARG, "fd_compute_init: NULL pointer");
  return dtype == FD_F64 ? launch_init<double>(*prm, mask, psi0, rho0, *out, as_stream(stream))
                         : launch_init<float>(*prm, mask, psi0, rho0, *out, as_stream(stream));
}

int fd_add_nonequilibrium(const fd_params* prm, int dtype, const uint16_t* mask, const fd_fields* fields,
                          void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(mask && fields_ok(fields), FD_ERR_ARG, "fd_add_nonequilibrium: NULL pointer");
  return dtype == FD_F64 ? launch_nonequilibrium<double>(*prm, mask, *fields, as_stream(stream))
                         : launch_nonequilibrium<float>(*prm, mask, *fields, as_stream(stream));
}

int fd_collide(const fd_params* prm, int dtype, const uint16_t* mask, const fd_fields* fields, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(mask && fields_ok(fields), FD_ERR_ARG, "fd_collide: NULL pointer");
  return dtype == FD_F64 ? launch_collide<double>(*prm, mask, *fields, as_stream(stream))
                         : launch_collide<float>(*prm, mask, *fields, as_stream(stream));
}

int fd_collision_term(const fd_params* prm, int dtype, int term, int j, const uint16_t* mask, const fd_fields* fields,
                      void* out, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(term >= FD_TERM_LARGE_F && term <= FD_TERM_G, FD_ERR_ARG, "unknown term %d", term);
  FD_REQUIRE(j >= 0 && j < 9, FD_ERR_ARG, "direction %d out of range", j);
  FD_REQUIRE(mask && out && fields_ok(fields), FD_ERR_ARG, "fd_collision_term: NULL pointer");
  return dtype == FD_F64 ? launch_term<double>(*prm, term, j, mask, *fields, out, as_stream(stream))
                         : launch_term<float>(*prm, term, j, mask, *fields, out, as_stream(stream));
}

int fd_stream(const fd_params* prm, int dtype, const void* src_f, const void* src_g, void* dst_f, void* dst_g,
              void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(src_f && src_g && dst_f && dst_g, FD_ERR_ARG, "fd_stream: NULL pointer");
  FD_REQUIRE(src_f != dst_f && src_g != dst_g, FD_ERR_ARG, "fd_stream: source and destination must differ");
  return dtype == FD_F64 ? launch_stream<double>(*prm, src_f, src_g, dst_f, dst_g, as_stream(stream))
                         : launch_stream<float>(*prm, src_f, src_g, dst_f, dst_g, as_stream(stream));
}

int fd_bounce_back(const fd_params* prm, int dtype, const uint16_t* mask, const void* f_behind, const void* g_behind,
                   void* f, void* g, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(mask && f_behind && g_behind && f && g, FD_ERR_ARG, "fd_bounce_back: NULL pointer");
  return dtype == FD_F64 ? launch_bb<double>(*prm, mask, f_behind, g_behind, f, g, as_stream(stream))
                         : launch_bb<float>(*prm, mask, f_behind, g_behind, f, g, as_stream(stream));
}

int fd_bottom_top_wall(int dtype, int rows, int cols, ptrdiff_t plane_stride, ptrdiff_t row_stride,
                       const void* f_behind, const void* g_behind, void* f, void* g, void* stream) {
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(rows >= 1 && cols >= 1, FD_ERR_SHAPE, "fd_bottom_top_wall: empty view");
  FD_REQUIRE(f_behind && g_behind && f && g, FD_ERR_ARG, "fd_bottom_top_wall: NULL pointer");
  return dtype == FD_F64
             ? launch_btw<double>(rows, cols, plane_stride, row_stride, f_behind, g_behind, f, g, as_stream(stream))
             : launch_btw<float>(rows, cols, plane_stride, row_stride, f_behind, g_behind, f, g, as_stream(stream));
}

int fd_boundary_fields(const fd_params* prm, int dtype, const uint16_t* mask, const void* psi, const void* np2,
                       void* side, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(mask && psi && np2 && side, FD_ERR_ARG, "fd_boundary_fields: NULL pointer");
  return dtype == FD_F64 ? launch_bfields<double>(*prm, mask, psi, np2, side, as_stream(stream))
                         : launch_bfields<float>(*prm, mask, psi, np2, side, as_stream(stream));
}

int fd_zou_he_inlet(const fd_params* prm, int dtype, void* f, void* g, const void* side, const double* inlet_ux,
                    void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(f && g && side && inlet_ux, FD_ERR_ARG, "fd_zou_he_inlet: NULL pointer");
  return dtype == FD_F64 ? launch_zou_he<double>(*prm, 0, f, g, side, inlet_ux, as_stream(stream))
                         : launch_zou_he<float>(*prm, 0, f, g, side, inlet_ux, as_stream(stream));
}

int fd_zou_he_outlet(const fd_params* prm, int dtype, void* f, void* g, const void* side, const double* inlet_ux,
                     void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(f && g && side && inlet_ux, FD_ERR_ARG, "fd_zou_he_outlet: NULL pointer");
  return dtype == FD_F64 ? launch_zou_he<double>(*prm, 1, f, g, side, inlet_ux, as_stream(stream))
                         : launch_zou_he<float>(*prm, 1, f, g, side, inlet_ux, as_stream(stream));
}

int fd_update_rho_psi(const fd_params* prm, int dtype, const uint16_t* mask, const fd_fields* fields, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(mask && fields_ok(fields), FD_ERR_ARG, "fd_update_rho_psi: NULL pointer");
  return dtype == FD_F64 ? launch_rho_psi<double>(*prm, mask, *fields, as_stream(stream))
                         : launch_rho_psi<float>(*prm, mask, *fields, as_stream(stream));
}

int fd_update_macros(const fd_params* prm, int dtype, const uint16_t* mask, const fd_fields* fields, void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(mask && fields_ok(fields), FD_ERR_ARG, "fd_update_macros: NULL pointer");
  return dtype == FD_F64 ? launch_macros<double>(*prm, mask, *fields, as_stream(stream))
                         : launch_macros<float>(*prm, mask, *fields, as_stream(stream));
}

int fd_field(const fd_params* prm, int dtype, int field_id, const uint16_t* mask, const fd_fields* fields, void* out,
             void* stream) {
  if (int r = check_params(prm)) return r;
  if (int r = check_dtype(dtype)) return r;
  FD_REQUIRE(field_id >= FD_FIELD_RHO && field_id <= FD_FIELD_PSI, FD_ERR_ARG, "unknown field %d", field_id);
  FD_REQUIRE(mask && out && fields_ok(fields), FD_ERR_ARG, "fd_field: NULL pointer");
  return dtype == FD_F64 ? launch_field<double>(*prm, field_id, mask, *fields, out, as_stream(stream))
                         : launch_field<float>(*prm, field_id, mask, *fields, out, as_stream(stream));
}

}  // extern "C"
