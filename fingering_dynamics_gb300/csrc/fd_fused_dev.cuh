// Fused step in deviation form with FP32 arithmetic (see fd_dev.cuh) and a
// storage type SF for the f deviations and g_1..g_8 (float, __half or
// __nv_bfloat16); g_0 is always stored in FP32.  Same pull / march / halo-lane
// structure as the exact kernel in fd_fused.cuh.
//
// Packed population buffer (one per ping-pong side), planes of P = H*W
// elements, each plane starting on a 256-byte boundary:
//   9 planes SF  : (f_i - w_i) * 2^s_f            i = 0..8
//   1 plane  f32 : g_0
//   8 planes SF  : g_i * 2^s_g                    i = 1..8
#pragma once

#include <type_traits>

#include "fd_dev.cuh"

namespace fd {

constexpr int kDevLanes = 30;
#ifndef FD_DEV_VEC
#define FD_DEV_VEC 2
#endif
#define FD_DEV_VEC_OF(SF) FD_DEV_VEC

inline size_t plane_bytes(size_t P, size_t elem) { return (P * elem + 255) / 256 * 256; }

// Device-side status word of the library's packed kernels:
//   bit 0 (kStatusWaitTimeout)  a bounded wait on an asynchronous copy gave up;
//   bit 1 (kStatusNonFinite)    a fused step met a non-finite density or psi in a
//                               fluid cell (numpy raises FloatingPointError there
//                               under the reference's np.seterr(all='raise'),
//                               fingering_periodic.py:496).
// The library is built without relocatable device code, so every translation
// unit that includes this header has its own copy, read and cleared through
// its own device_error_word(); fd_device_status() combines the copies.
constexpr unsigned kStatusWaitTimeout = 1u;
constexpr unsigned kStatusNonFinite = 2u;
__device__ unsigned int g_fd_device_error = 0;

namespace {
inline int device_error_word(unsigned* out, bool clear) {
  if (cudaMemcpyFromSymbol(out, g_fd_device_error, sizeof(unsigned)) != cudaSuccess) return FD_ERR_CUDA;
  if (clear) {
    const unsigned zero = 0;
    if (cudaMemcpyToSymbol(g_fd_device_error, &zero, sizeof(unsigned)) != cudaSuccess) return FD_ERR_CUDA;
  }
  return FD_OK;
}
}  // namespace

// true if rho or psi of a fluid cell is not finite (NaN or +-inf)
__device__ __forceinline__ bool nonfinite_cell(float rho, float psi) { return !(fabsf(rho) + fabsf(psi) < INFINITY); }

template <typename SF>
struct DevArgs {
  DevCoef c;
  int H, W, variant, nchunks, nstrips, R;
  size_t P, pstride_f;  // plane size and plane stride (elements of SF)
  const uint16_t* __restrict__ mask;
  const double* __restrict__ inlet_ux;
  const SF* __restrict__ src_f;
  const float* __restrict__ src_g0;
  const SF* __restrict__ src_gi;  // plane i>=1 at src_gi + (i-1)*pstride_f
  SF* __restrict__ dst_f;
  float* __restrict__ dst_g0;
  SF* __restrict__ dst_gi;
  const float* __restrict__ side_in;
  float* __restrict__ side_out;
  uint32_t seed;  // stochastic rounding: sr_hash of the step's seed
  // where a non-finite cell is reported: a batch member's status word (set to
  // 1; the batched kernel skips the member's tiles from then on), or null for
  // the unit's device status word (bit kStatusNonFinite)
  unsigned* status;
};

template <typename SF>
__device__ __forceinline__ void report_nonfinite(const DevArgs<SF>& a) {
  if (a.status) atomicOr(a.status, 1u);
  else atomicOr(&g_fd_device_error, kStatusNonFinite);
}

template <typename S, int VEC>
__device__ __forceinline__ void ld_conv(const S* __restrict__ p, float scale, float (&out)[VEC]) {
  S v[VEC];
  ld_vec<S, VEC>(p, v);
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    if constexpr (std::is_same_v<S, float>) out[k] = v[k];
    else out[k] = to_f<S>(v[k]) * scale;
  }
}

template <typename S, int VEC>
__device__ __forceinline__ void st_conv(S* __restrict__ p, float scale, const float (&in)[VEC]) {
  S v[VEC];
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    if constexpr (std::is_same_v<S, float>) v[k] = in[k];
    else v[k] = from_f<S>(in[k] * scale);
  }
  st_vec<S, VEC>(p, v);
}

// st_conv with stochastic rounding; rs[k] is the random state of cell k
template <typename S, int VEC>
__device__ __forceinline__ void st_conv_sr(S* __restrict__ p, float scale, const float (&in)[VEC], uint32_t (&rs)[VEC]) {
  S v[VEC];
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    rs[k] = sr_next(rs[k]);
    v[k] = from_f_sr<S>(in[k] * scale, rs[k]);
  }
  st_vec<S, VEC>(p, v);
}

template <typename S>
__device__ __forceinline__ float ld_one(const S* __restrict__ p, float scale) {
  if constexpr (std::is_same_v<S, float>) return __ldg(p);
  else return to_f<S>(p[0]) * scale;
}

// pull one plane into out[] with the x shift of direction I (warp shuffles)
template <int I, typename S, int VEC>
__device__ __forceinline__ void pull_plane(const S* __restrict__ plane, int H, int W, int y, int xw, float scale,
                                           float (&out)[VEC]) {
  constexpr int ex = ex_of(I), ey = ey_of(I);
  const int ys = wrap(y - ey, H);
  float v[VEC];
  ld_conv<S, VEC>(plane + (size_t)ys * W + xw, scale, v);
  if constexpr (ex == 0) {
#pragma unroll
    for (int k = 0; k < VEC; ++k) out[k] = v[k];
  } else if constexpr (ex == 1) {
    const float l = __shfl_up_sync(0xffffffffu, v[VEC - 1], 1);
    out[0] = l;
#pragma unroll
    for (int k = 1; k < VEC; ++k) out[k] = v[k - 1];
  } else {
    const float r = __shfl_down_sync(0xffffffffu, v[0], 1);
#pragma unroll
    for (int k = 0; k < VEC - 1; ++k) out[k] = v[k + 1];
    out[VEC - 1] = r;
  }
}

template <typename SF, int VEC>
__device__ __forceinline__ void pull_f_row(const DevArgs<SF>& a, int y, int xw, const uint16_t (&mb)[VEC],
                                           float (&f)[9][VEC]) {
  const SF* b = a.src_f;
  const size_t ps = a.pstride_f;
  const float s = a.c.inv_sf;
  pull_plane<0>(b, a.H, a.W, y, xw, s, f[0]);
  pull_plane<1>(b + ps, a.H, a.W, y, xw, s, f[1]);
  pull_plane<2>(b + 2 * ps, a.H, a.W, y, xw, s, f[2]);
  pull_plane<3>(b + 3 * ps, a.H, a.W, y, xw, s, f[3]);
  pull_plane<4>(b + 4 * ps, a.H, a.W, y, xw, s, f[4]);
  pull_plane<5>(b + 5 * ps, a.H, a.W, y, xw, s, f[5]);
  pull_plane<6>(b + 6 * ps, a.H, a.W, y, xw, s, f[6]);
  pull_plane<7>(b + 7 * ps, a.H, a.W, y, xw, s, f[7]);
  pull_plane<8>(b + 8 * ps, a.H, a.W, y, xw, s, f[8]);
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    const unsigned bits = mb[k] & 0xFFu;
    if (bits) {
      const size_t q = (size_t)y * a.W + xw + k;
#pragma unroll
      for (int i = 1; i < 9; ++i)
        if (bits & (1u << (i - 1))) f[i][k] = ld_one(b + (size_t)opp_of(i) * ps + q, s);
    }
  }
}

template <typename SF, int VEC>
__device__ __forceinline__ void pull_g_row(const DevArgs<SF>& a, int y, int xw, const uint16_t (&mb)[VEC],
                                           float (&g)[9][VEC]) {
  const SF* b = a.src_gi;
  const size_t ps = a.pstride_f;
  const float s = a.c.inv_sg;
  pull_plane<0>(a.src_g0, a.H, a.W, y, xw, 1.0f, g[0]);
  pull_plane<1>(b, a.H, a.W, y, xw, s, g[1]);
  pull_plane<2>(b + ps, a.H, a.W, y, xw, s, g[2]);
  pull_plane<3>(b + 2 * ps, a.H, a.W, y, xw, s, g[3]);
  pull_plane<4>(b + 3 * ps, a.H, a.W, y, xw, s, g[4]);
  pull_plane<5>(b + 4 * ps, a.H, a.W, y, xw, s, g[5]);
  pull_plane<6>(b + 5 * ps, a.H, a.W, y, xw, s, g[6]);
  pull_plane<7>(b + 6 * ps, a.H, a.W, y, xw, s, g[7]);
  pull_plane<8>(b + 7 * ps, a.H, a.W, y, xw, s, g[8]);
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    const unsigned bits = mb[k] & 0xFFu;
    if (bits) {
      const size_t q = (size_t)y * a.W + xw + k;
#pragma unroll
      for (int i = 1; i < 9; ++i)
        if (bits & (1u << (i - 1))) g[i][k] = ld_one(b + (size_t)(opp_of(i) - 1) * ps + q, s);
    }
  }
}

// psi of the row's cells: the pair (hi, lo) of dev_psi_pair for FP32 storage,
// else (psi, 0) (see the staged kernel's psi_paired).
template <typename SF, int VEC>
__device__ __forceinline__ void g_row_dev(const DevArgs<SF>& a, int y, int x0, int xw, uint16_t (&mb)[VEC],
                                          float (&g)[9][VEC], float2 (&psi)[VEC]) {
  ld_vec<uint16_t, VEC>(a.mask + (size_t)y * a.W + xw, mb);
  pull_g_row<SF, VEC>(a, y, xw, mb, g);
  if (x0 == 0) {
    float gc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gc[i] = g[i][0];
    dev_zou_he_g(a.c, a.variant, a.H, a.W, 0, y, gc);
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i][0] = gc[i];
  }
  if (x0 == a.W - VEC) {
    float gc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gc[i] = g[i][VEC - 1];
    dev_zou_he_g(a.c, a.variant, a.H, a.W, a.W - 1, y, gc);
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i][VEC - 1] = gc[i];
  }
#pragma unroll
  for (int k = 0; k < VEC; ++k) {
    const int x = x0 + k;
    float gc[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) gc[i] = g[i][k];
    float2 s;
    if constexpr (std::is_same_v<SF, float>) {
      s = dev_psi_pair(gc);
    } else {
      const float S = ((gc[1] + gc[2]) + (gc[3] + gc[4])) + ((gc[5] + gc[6]) + (gc[7] + gc[8]));
      s = make_float2(gc[0] + S, 0.0f);
    }
    psi[k] = (x < 0) ? make_float2(1.0f, 0.0f)
                     : (x >= a.W) ? make_float2(-1.0f, 0.0f)
                                  : ((mb[k] & SOLID) ? make_float2(a.c.psi_wall, 0.0f) : s);
  }
}

template <typename SF>
__device__ __forceinline__ float dev_rho_inlet_row(const DevArgs<SF>& a, int yn) {
  // pulled deviations 0,2,4,3,6,7 of cell (0, yn) (bounce-back links applied)
  const size_t q = (size_t)yn * a.W;
  const unsigned bits = a.mask[q] & 0xFFu;
  float d[9];
  const int dirs[6] = {0, 2, 4, 3, 6, 7};
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const int i = dirs[t];
    const SF* src;
    if (i > 0 && (bits & (1u << (i - 1)))) src = a.src_f + (size_t)opp_of(i) * a.pstride_f + q;
    else src = a.src_f + (size_t)i * a.pstride_f + (size_t)wrap(yn - ey_of(i), a.H) * a.W + wrap(-ex_of(i), a.W);
    d[i] = ld_one(src, a.c.inv_sf);
  }
  d[1] = d[5] = d[8] = 0.0f;
  return dev_inlet_drho(d, (float)a.inlet_ux[yn], a.side_in[0 * a.H + yn], a.side_in[2 * a.H + yn]);
}

template <typename SF, int VEC, int K>
__device__ __forceinline__ void dev_boundary_cell(const DevArgs<SF>& a, int y, int x, float (&f)[9][VEC],
                                                  const DevStencil (&st)[VEC]) {
  const int o = (x == 0) ? 0 : 3;
  float drho_nb = 0.0f;
  if (a.variant == FD_VARIANT_WALLS && x == 0 && (y == 0 || y == a.H - 1))
    drho_nb = dev_rho_inlet_row(a, y == 0 ? 1 : a.H - 2);
  float fc[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) fc[i] = f[i][K];
  dev_zou_he_f(a.c, a.variant, a.H, a.W, x, y, fc, (float)a.inlet_ux[y], a.side_in[(o + 0) * a.H + y],
               a.side_in[(o + 1) * a.H + y], a.side_in[(o + 2) * a.H + y], drho_nb);
#pragma unroll
  for (int i = 0; i < 9; ++i) f[i][K] = fc[i];
  a.side_out[(o + 0) * a.H + y] = st[K].gx;
  a.side_out[(o + 1) * a.H + y] = st[K].gy;
  a.side_out[(o + 2) * a.H + y] = dev_mu(a.c, st[K]);
}

template <int VEC>
__device__ __forceinline__ void extend_f(const float2 (&p)[VEC], float2 (&e)[VEC + 2]) {
  e[0] = make_float2(__shfl_up_sync(0xffffffffu, p[VEC - 1].x, 1), __shfl_up_sync(0xffffffffu, p[VEC - 1].y, 1));
#pragma unroll
  for (int k = 0; k < VEC; ++k) e[k + 1] = p[k];
  e[VEC + 1] = make_float2(__shfl_down_sync(0xffffffffu, p[0].x, 1), __shfl_down_sync(0xffffffffu, p[0].y, 1));
}

#ifndef FD_DEV_MINB
#define FD_DEV_MINB 4
#endif
#ifndef FD_DEV_PREFETCH
#define FD_DEV_PREFETCH 2
#endif

// Asynchronous L2 prefetch of one row segment of every plane the warp will
// read `dist` rows from now: one bulk prefetch per plane, issued by lane 0, so
// that the demand loads of later rows find their lines in L2.
template <typename SF>
__device__ __forceinline__ void prefetch_rows(const DevArgs<SF>& a, int lane, int chunk, int yf, int yg) {
  if (lane != 0) return;
  constexpr int VB = 16;  // alignment of a bulk prefetch, bytes
  const int x_lo = max(chunk * kDevLanes * FD_DEV_VEC_OF(SF) - FD_DEV_VEC_OF(SF), 0);
  const int x_hi = min((chunk + 1) * kDevLanes * FD_DEV_VEC_OF(SF) + FD_DEV_VEC_OF(SF), a.W);
  auto issue = [&](const void* p, int nbytes) {
    const uintptr_t lo = (uintptr_t)p & ~(uintptr_t)(VB - 1);
    const uintptr_t hi = ((uintptr_t)p + nbytes + VB - 1) & ~(uintptr_t)(VB - 1);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(lo), "r"((unsigned)(hi - lo)) : "memory");
  };
  const size_t rf = (size_t)yf * a.W + x_lo, rg = (size_t)yg * a.W + x_lo;
  const int nf = (x_hi - x_lo) * (int)sizeof(SF);
#pragma unroll
  for (int i = 0; i < 9; ++i) issue(a.src_f + i * a.pstride_f + rf, nf);
  issue(a.src_g0 + rg, (x_hi - x_lo) * 4);
#pragma unroll
  for (int i = 0; i < 8; ++i) issue(a.src_gi + i * a.pstride_f + rg, nf);
}

template <typename SF, int VEC, bool STOCH>
__global__ void __launch_bounds__(128, FD_DEV_MINB) k_fused_dev(const DevArgs<SF> a) {
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (warp >= a.nchunks * a.nstrips) return;
  const int chunk = warp % a.nchunks, strip = warp / a.nchunks;
  const int x0 = (chunk * kDevLanes + lane - 1) * VEC;
  const int xw = ((x0 % a.W) + a.W) % a.W;
  const bool owned = lane >= 1 && lane <= kDevLanes && x0 >= 0 && x0 < a.W;
  const int y0 = strip * a.R, y1 = min(y0 + a.R, a.H);
  const bool walls = a.variant == FD_VARIANT_WALLS;

  float gC[9][VEC], gN[9][VEC];
  float2 Pm[VEC], Pc[VEC], Pn[VEC];
  uint16_t mC[VEC], mN[VEC];
  bool bad = false;  // a fluid cell with a non-finite rho or psi

  if (walls && y0 == 0) {
#pragma unroll
    for (int k = 0; k < VEC; ++k) Pm[k] = make_float2(a.c.psi_wall, 0.0f);
  } else {
    g_row_dev<SF, VEC>(a, wrap(y0 - 1, a.H), x0, xw, mN, gN, Pm);
  }
  g_row_dev<SF, VEC>(a, y0, x0, xw, mC, gC, Pc);

  for (int y = y0; y < y1; ++y) {
    if (FD_DEV_PREFETCH > 0 && y + FD_DEV_PREFETCH < y1)
      prefetch_rows(a, lane, chunk, wrap(y + 1 + FD_DEV_PREFETCH, a.H), wrap(y + 2 + FD_DEV_PREFETCH, a.H));
    if (walls && y + 1 >= a.H) {
#pragma unroll
      for (int k = 0; k < VEC; ++k) Pn[k] = make_float2(a.c.psi_wall, 0.0f);
    } else {
      g_row_dev<SF, VEC>(a, wrap(y + 1, a.H), x0, xw, mN, gN, Pn);
    }
    float2 em[VEC + 2], ec[VEC + 2], en[VEC + 2];
    extend_f<VEC>(Pm, em);
    extend_f<VEC>(Pc, ec);
    extend_f<VEC>(Pn, en);
    DevStencil st[VEC];
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
      if constexpr (std::is_same_v<SF, float>)
        st[k] = dev_stencil_pair(ec[k + 1], ec[k + 2], ec[k], en[k + 1], em[k + 1], en[k + 2], en[k], em[k + 2],
                                 em[k]);
      else
        st[k] = dev_stencil(ec[k + 1].x, ec[k + 2].x, ec[k].x, en[k + 1].x, em[k + 1].x, en[k + 2].x, en[k].x,
                            em[k + 2].x, em[k].x);
    }
    float f[9][VEC];
    pull_f_row<SF, VEC>(a, y, xw, mC, f);
    if (owned && x0 == 0) dev_boundary_cell<SF, VEC, 0>(a, y, 0, f, st);
    if (owned && x0 == a.W - VEC) dev_boundary_cell<SF, VEC, VEC - 1>(a, y, a.W - 1, f, st);
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
      if (!(mC[k] & SOLID)) {
        float fc[9], gc[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) { fc[i] = f[i][k]; gc[i] = gC[i][k]; }
        const DevMacro m = dev_macros(a.c, fc, st[k]);
        bad |= nonfinite_cell(m.rho, m.psi);
        dev_collide(a.c, m, fc, gc);
#pragma unroll
        for (int i = 0; i < 9; ++i) { f[i][k] = fc[i]; gC[i][k] = gc[i]; }
      }
    }
    if (owned) {
      const size_t row = (size_t)y * a.W + x0;
      if constexpr (STOCH) {
        uint32_t rs[VEC];
#pragma unroll
        for (int k = 0; k < VEC; ++k) rs[k] = sr_hash((uint32_t)(row + k) ^ a.seed);
#pragma unroll
        for (int i = 0; i < 9; ++i) st_conv_sr<SF, VEC>(a.dst_f + i * a.pstride_f + row, a.c.sf, f[i], rs);
        st_conv<float, VEC>(a.dst_g0 + row, 1.0f, gC[0]);
#pragma unroll
        for (int i = 1; i < 9; ++i) st_conv_sr<SF, VEC>(a.dst_gi + (i - 1) * a.pstride_f + row, a.c.sg, gC[i], rs);
      } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) st_conv<SF, VEC>(a.dst_f + i * a.pstride_f + row, a.c.sf, f[i]);
        st_conv<float, VEC>(a.dst_g0 + row, 1.0f, gC[0]);
#pragma unroll
        for (int i = 1; i < 9; ++i) st_conv<SF, VEC>(a.dst_gi + (i - 1) * a.pstride_f + row, a.c.sg, gC[i]);
      }
    }
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
      Pm[k] = Pc[k];
      Pc[k] = Pn[k];
      mC[k] = mN[k];
#pragma unroll
      for (int i = 0; i < 9; ++i) gC[i][k] = gN[i][k];
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) report_nonfinite(a);
}

// ---- pack / unpack between the reference layout (18 planes of T) and the
// packed deviation layout ------------------------------------------------------
template <typename T, typename SF>
__global__ void k_pack(size_t P, size_t pstride, DevCoef c, const T* __restrict__ src, SF* __restrict__ f,
                       float* __restrict__ g0, SF* __restrict__ gi) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
#pragma unroll
  for (int i = 0; i < 9; ++i) f[i * pstride + q] = from_f<SF>(((float)src[i * P + q] - c.w[i]) * c.sf);
  g0[q] = (float)src[9 * P + q];
#pragma unroll
  for (int i = 1; i < 9; ++i) gi[(i - 1) * pstride + q] = from_f<SF>((float)src[(9 + i) * P + q] * c.sg);
}

template <typename T, typename SF>
__global__ void k_unpack(size_t P, size_t pstride, DevCoef c, const SF* __restrict__ f, const float* __restrict__ g0,
                         const SF* __restrict__ gi, T* __restrict__ dst) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
#pragma unroll
  for (int i = 0; i < 9; ++i) dst[i * P + q] = (T)(to_f<SF>(f[i * pstride + q]) * c.inv_sf + c.w[i]);
  dst[9 * P + q] = (T)g0[q];
#pragma unroll
  for (int i = 1; i < 9; ++i) dst[(9 + i) * P + q] = (T)(to_f<SF>(gi[(i - 1) * pstride + q]) * c.inv_sg);
}

template <typename SF>
struct PackedLayout {
  size_t P, pstride;
  size_t off_f, off_g0, off_gi, total;
};

template <typename SF>
inline PackedLayout<SF> packed_layout(int H, int W) {
  PackedLayout<SF> L;
  L.P = (size_t)H * W;
  const size_t bf = plane_bytes(L.P, sizeof(SF));
  L.pstride = bf / sizeof(SF);
  L.off_f = 0;
  L.off_g0 = 9 * bf;
  L.off_gi = L.off_g0 + plane_bytes(L.P, sizeof(float));
  L.total = L.off_gi + 8 * bf;
  return L;
}

template <typename SF, int VEC, bool STOCH>
int launch_fused_dev(const fd_params& p, const DevCoef& c, const uint16_t* mask, const double* inlet_ux, char* pa,
                     char* pb, float* sa, float* sb, int nsteps, int R, uint32_t seed, cudaStream_t st) {
  const PackedLayout<SF> L = packed_layout<SF>(p.H, p.W);
  DevArgs<SF> a;
  a.c = c;
  a.H = p.H;
  a.W = p.W;
  a.variant = p.variant;
  a.nchunks = (p.W / VEC + kDevLanes - 1) / kDevLanes;
  a.R = R;
  a.nstrips = (p.H + R - 1) / R;
  a.P = L.P;
  a.pstride_f = L.pstride;
  a.mask = mask;
  a.inlet_ux = inlet_ux;
  a.status = nullptr;
  const long long warps = (long long)a.nchunks * a.nstrips;
  const unsigned blocks = (unsigned)((warps * 32 + 127) / 128);
  for (int s = 0; s < nsteps; ++s) {
    char* src = (s % 2 == 0) ? pa : pb;
    char* dst = (s % 2 == 0) ? pb : pa;
    a.src_f = reinterpret_cast<const SF*>(src + L.off_f);
    a.src_g0 = reinterpret_cast<const float*>(src + L.off_g0);
    a.src_gi = reinterpret_cast<const SF*>(src + L.off_gi);
    a.dst_f = reinterpret_cast<SF*>(dst + L.off_f);
    a.dst_g0 = reinterpret_cast<float*>(dst + L.off_g0);
    a.dst_gi = reinterpret_cast<SF*>(dst + L.off_gi);
    a.side_in = (s % 2 == 0) ? sa : sb;
    a.side_out = (s % 2 == 0) ? sb : sa;
    a.seed = sr_hash(seed + (uint32_t)s);
    k_fused_dev<SF, VEC, STOCH><<<blocks, 128, 0, st>>>(a);
  }
  return cudaGetLastError() == cudaSuccess ? FD_OK : FD_ERR_CUDA;
}

template <typename T, typename SF>
int launch_pack(const fd_params& p, const DevCoef& c, const void* src, char* dst, cudaStream_t st) {
  const PackedLayout<SF> L = packed_layout<SF>(p.H, p.W);
  k_pack<T, SF><<<(unsigned)((L.P + 255) / 256), 256, 0, st>>>(
      L.P, L.pstride, c, (const T*)src, reinterpret_cast<SF*>(dst + L.off_f), reinterpret_cast<float*>(dst + L.off_g0),
      reinterpret_cast<SF*>(dst + L.off_gi));
  return cudaGetLastError() == cudaSuccess ? FD_OK : FD_ERR_CUDA;
}

template <typename T, typename SF>
int launch_unpack(const fd_params& p, const DevCoef& c, const char* src, void* dst, cudaStream_t st) {
  const PackedLayout<SF> L = packed_layout<SF>(p.H, p.W);
  k_unpack<T, SF><<<(unsigned)((L.P + 255) / 256), 256, 0, st>>>(
      L.P, L.pstride, c, reinterpret_cast<const SF*>(src + L.off_f), reinterpret_cast<const float*>(src + L.off_g0),
      reinterpret_cast<const SF*>(src + L.off_gi), (T*)dst);
  return cudaGetLastError() == cudaSuccess ? FD_OK : FD_ERR_CUDA;
}

}  // namespace fd
