// Training and inference kernels of the learned surrogate (include/fdsurrogate.h).
//
// Convolutions are implicit GEMMs on the tensor cores with bfloat16 operands
// and FP32 accumulation (mma.sync m16n8k16; operand tiles staged in shared
// memory by cp.async, fragments loaded with ldmatrix):
//   forward / data gradient: M = pixels, N = output channels, K = 9 x input
//     channels; a CTA computes 64 pixels x BN channels, marching over the input
//     channels in chunks of BK and, within a chunk, over the nine taps
//     (their input rows overlap, so the copies go through L1), double-buffered;
//   weight gradient: M = output channels, N = input channels of one tap, K =
//     pixels, split over pixel ranges into FP32 partials that one pass adds in
//     a fixed order.
// The network around them is defined in fingering_dynamics_gb300/surrogate.py.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fdsurrogate.h"
#include "fd_host.h"

namespace sg {
namespace {

using bf16 = __nv_bfloat16;
constexpr int kThreads = 128;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// 16-byte global -> shared copy; src_bytes = 0 writes zeros (padding)
__device__ __forceinline__ void cp16(void* dst, const void* src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
// the same through L1: the nine taps of a chunk re-read neighbouring pixels
__device__ __forceinline__ void cp16_l1(void* dst, const void* src, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(smem_u32(p)));
}

// D += A (16x16, row) * B (16x8, col), bfloat16 in, FP32 accumulate
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// GELU, tanh form: 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))
__device__ __forceinline__ float gelu_f(float z) {
  const float u = 0.7978845608028654f * fmaf(0.044715f * z * z, z, z);
  return 0.5f * z * (1.0f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad_f(float z) {
  const float u = 0.7978845608028654f * fmaf(0.044715f * z * z, z, z);
  const float t = tanhf(u);
  const float du = 0.7978845608028654f * fmaf(3.0f * 0.044715f, z * z, 1.0f);
  return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * du;
}

// ---------------------------------------------------------------------------
// forward convolution (also the data gradient with flipped weights)
// ---------------------------------------------------------------------------
template <int BN, int BK, int WM, int WN>
struct ConvCfg {
  static constexpr int BM = 64;
  static constexpr int TM = BM / WM, TN = BN / WN;
  static constexpr int MT = TM / 16, NT = TN / 8;
  static constexpr int LDS = BK + 8;                 // shared row stride (elements): conflict-free ldmatrix
  static constexpr int VPR = BK / 8;                 // 16-byte vectors per row of a chunk
  static constexpr int A_VEC = BM * VPR, B_VEC = BN * VPR;
  static_assert(WM * WN == 4, "four warps");
  static_assert(MT >= 1 && NT % 2 == 0 && TM % 16 == 0 && TN % 16 == 0, "warp tile");
};

template <int BN, int BK, int WM, int WN>
__global__ void __launch_bounds__(kThreads) k_conv3x3(const bf16* __restrict__ x, int N, int H, int W, int Cin,
                                                      const bf16* __restrict__ w, const float* __restrict__ bias,
                                                      int Cout, int act, bf16* __restrict__ z, bf16* __restrict__ y) {
  using C = ConvCfg<BN, BK, WM, WN>;
  __shared__ __align__(16) bf16 As[2][C::BM * C::LDS];
  __shared__ __align__(16) bf16 Bs[2][BN * C::LDS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp / WN, wn = warp % WN;
  const long long M = (long long)N * H * W;
  const long long m0 = (long long)blockIdx.x * C::BM;
  const int co0 = blockIdx.y * BN;
  const int cchunks = Cin / BK, nk = 9 * cchunks;

  // the pixels whose A vectors this thread copies (fixed over the K loop):
  // their address at the centre tap, their shared-memory slot and a 9-bit
  // mask of the taps that fall inside the image
  constexpr int A_PER = (C::A_VEC + kThreads - 1) / kThreads;
  const bf16* a_base[A_PER];
  uint32_t a_valid[A_PER];
  int a_soff[A_PER];
#pragma unroll
  for (int i = 0; i < A_PER; ++i) {
    const int v = tid + i * kThreads;
    const int row = v / C::VPR, sub = v % C::VPR;
    const long long p = m0 + row;
    a_soff[i] = row * C::LDS + sub * 8;
    a_base[i] = x;
    a_valid[i] = 0u;
    if (v < C::A_VEC && p < M) {
      const int rem = (int)(p % ((long long)H * W));
      const int yy = rem / W, xx = rem % W;
      a_base[i] = x + p * Cin + sub * 8;
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int ty = yy + t / 3 - 1, tx = xx + t % 3 - 1;
        if (ty >= 0 && ty < H && tx >= 0 && tx < W) a_valid[i] |= 1u << t;
      }
    }
  }

  // K order: input-channel chunk major, the nine taps of a chunk back to back
  auto load_chunk = [&](int kc, int stage) {
    const int tap = kc % 9, ci0 = (kc / 9) * BK;
    const long long toff = ((long long)(tap / 3 - 1) * W + (tap % 3 - 1)) * Cin + ci0;
#pragma unroll
    for (int i = 0; i < A_PER; ++i) {
      const bool ok = (a_valid[i] >> tap) & 1u;
      if (tid + i * kThreads < C::A_VEC) cp16_l1(&As[stage][a_soff[i]], ok ? a_base[i] + toff : x, ok ? 16 : 0);
    }
    for (int v = tid; v < C::B_VEC; v += kThreads) {
      const int r = v / C::VPR, sub = v % C::VPR;
      const bf16* src = w + ((long long)(co0 + r) * 9 + tap) * Cin + ci0 + sub * 8;
      cp16(&Bs[stage][r * C::LDS + sub * 8], src, 16);
    }
  };

  float acc[C::MT][C::NT][4];
#pragma unroll
  for (int a = 0; a < C::MT; ++a)
#pragma unroll
    for (int b = 0; b < C::NT; ++b)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[a][b][k] = 0.0f;

  load_chunk(0, 0);
  cp_commit();
  for (int kc = 0; kc < nk; ++kc) {
    const int st = kc & 1;
    if (kc + 1 < nk) load_chunk(kc + 1, st ^ 1);
    cp_commit();
    cp_wait<1>();
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < BK / 16; ++ks) {
      uint32_t af[C::MT][4], bfr[C::NT][2];
#pragma unroll
      for (int mt = 0; mt < C::MT; ++mt) {
        const int r = wm * C::TM + mt * 16 + (lane & 15);
        ldsm_x4(af[mt], &As[st][r * C::LDS + ks * 16 + (lane >> 4) * 8]);
      }
      // two n8 fragments per ldmatrix: lanes 16..31 address the second
#pragma unroll
      for (int nt = 0; nt < C::NT; nt += 2) {
        uint32_t r4[4];
        const int r = wn * C::TN + nt * 8 + (lane & 7) + ((lane >> 4) << 3);
        ldsm_x4(r4, &Bs[st][r * C::LDS + ks * 16 + ((lane >> 3) & 1) * 8]);
        bfr[nt][0] = r4[0];
        bfr[nt][1] = r4[1];
        bfr[nt + 1][0] = r4[2];
        bfr[nt + 1][1] = r4[3];
      }
#pragma unroll
      for (int mt = 0; mt < C::MT; ++mt)
#pragma unroll
        for (int nt = 0; nt < C::NT; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt]);
    }
    __syncthreads();
  }

  // epilogue: bias, activation, bfloat16 pairs
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mt = 0; mt < C::MT; ++mt) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const long long p = m0 + wm * C::TM + mt * 16 + g + half * 8;
      if (p >= M) continue;
#pragma unroll
      for (int nt = 0; nt < C::NT; ++nt) {
        const int co = co0 + wn * C::TN + nt * 8 + 2 * t;
        float v0 = acc[mt][nt][half * 2 + 0], v1 = acc[mt][nt][half * 2 + 1];
        if (bias) {
          v0 += bias[co];
          v1 += bias[co + 1];
        }
        const size_t o = (size_t)p * Cout + co;
        if (z) *reinterpret_cast<__nv_bfloat162*>(z + o) = __floats2bfloat162_rn(v0, v1);
        if (act == SG_ACT_GELU) {
          v0 = gelu_f(v0);
          v1 = gelu_f(v1);
        }
        if (y) *reinterpret_cast<__nv_bfloat162*>(y + o) = __floats2bfloat162_rn(v0, v1);
      }
    }
  }
}

template <int BN, int BK, int WM, int WN>
void launch_conv(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
                 bf16* z, bf16* y, cudaStream_t s) {
  const long long M = (long long)N * H * W;
  dim3 grid((unsigned)((M + 63) / 64), (unsigned)(Cout / BN));
  k_conv3x3<BN, BK, WM, WN><<<grid, kThreads, 0, s>>>(x, N, H, W, Cin, w, b, Cout, act, z, y);
}

template <int BK>
void conv_bk(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act, bf16* z,
             bf16* y, cudaStream_t s) {
  if (Cout % 64 == 0) launch_conv<64, BK, 2, 2>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  else if (Cout % 32 == 0) launch_conv<32, BK, 2, 2>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  else launch_conv<16, BK, 4, 1>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
}

// ---------------------------------------------------------------------------
// weight gradient
// ---------------------------------------------------------------------------
template <int BM, int BN>
struct WgCfg {
  static constexpr int BK = 64;                              // pixels per chunk
  static constexpr int WM = BM >= 32 ? 2 : 1;
  static constexpr int WN_MAX = 4 / WM;
  static constexpr int WN = (BN / 8) < WN_MAX ? (BN / 8) : WN_MAX;
  static constexpr int TM = BM / WM, TN = BN / WN;
  static constexpr int MT = TM / 16, NT = TN / 8;
  static constexpr int LDA = BM + 8, LDB = BN + 8;
  static constexpr int AV = BK * BM / 8, BV = BK * BN / 8;  // 16-byte vectors per chunk
  static_assert(MT >= 1 && NT >= 1, "warp tile");
};

template <int BM, int BN>
__global__ void __launch_bounds__(kThreads) k_wgrad(const bf16* __restrict__ x, const bf16* __restrict__ dz, int N,
                                                    int H, int W, int Cin, int Cout, int splits, long long chunk,
                                                    float* __restrict__ partial) {
  using C = WgCfg<BM, BN>;
  __shared__ __align__(16) bf16 As[2][C::BK * C::LDA];  // [pixel][co]
  __shared__ __align__(16) bf16 Bs[2][C::BK * C::LDB];  // [pixel][ci]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int co0 = blockIdx.x * BM, ci0 = blockIdx.y * BN;
  const int tap = blockIdx.z % 9, split = blockIdx.z / 9;
  const int ky = tap / 3 - 1, kx = tap % 3 - 1;
  const long long M = (long long)N * H * W;
  const long long p0 = (long long)split * chunk, p1 = min(M, p0 + chunk);
  const bool active = warp < C::WM * C::WN;
  const int wm = warp / C::WN, wn = warp % C::WN;

  // Each thread copies fixed rows of every chunk: A rows are dz pixels, B
  // rows x pixels shifted by the tap.  Their pixel index advances by BK per
  // chunk; the (y, x) of the B rows is carried along without divisions.
  constexpr int A_PER = (C::AV + kThreads - 1) / kThreads, B_PER = (C::BV + kThreads - 1) / kThreads;
  long long a_p[A_PER], b_p[B_PER];
  int b_y[B_PER], b_x[B_PER];
#pragma unroll
  for (int i = 0; i < A_PER; ++i) a_p[i] = p0 + (tid + i * kThreads) / (BM / 8);
#pragma unroll
  for (int i = 0; i < B_PER; ++i) {
    b_p[i] = p0 + (tid + i * kThreads) / (BN / 8);
    const int rem = (int)(b_p[i] % ((long long)H * W));
    b_y[i] = rem / W;
    b_x[i] = rem % W;
  }
  const long long toff = ((long long)ky * W + kx) * Cin + ci0;

  auto load_chunk = [&](int st) {
#pragma unroll
    for (int i = 0; i < A_PER; ++i) {
      const int v = tid + i * kThreads;
      if (v < C::AV) {
        const int r = v / (BM / 8), sub = v % (BM / 8);
        const bool ok = a_p[i] < p1;
        cp16(&As[st][r * C::LDA + sub * 8], ok ? dz + a_p[i] * Cout + co0 + sub * 8 : dz, ok ? 16 : 0);
      }
    }
#pragma unroll
    for (int i = 0; i < B_PER; ++i) {
      const int v = tid + i * kThreads;
      if (v < C::BV) {
        const int r = v / (BN / 8), sub = v % (BN / 8);
        const int yy = b_y[i] + ky, xx = b_x[i] + kx;
        const bool ok = b_p[i] < p1 && yy >= 0 && yy < H && xx >= 0 && xx < W;
        cp16(&Bs[st][r * C::LDB + sub * 8], ok ? x + b_p[i] * Cin + toff + sub * 8 : x, ok ? 16 : 0);
      }
    }
  };
  auto advance = [&]() {
#pragma unroll
    for (int i = 0; i < A_PER; ++i) a_p[i] += C::BK;
#pragma unroll
    for (int i = 0; i < B_PER; ++i) {
      b_p[i] += C::BK;
      b_x[i] += C::BK;
      while (b_x[i] >= W) {
        b_x[i] -= W;
        if (++b_y[i] == H) b_y[i] = 0;
      }
    }
  };

  float acc[C::MT][C::NT][4];
#pragma unroll
  for (int a = 0; a < C::MT; ++a)
#pragma unroll
    for (int b = 0; b < C::NT; ++b)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[a][b][k] = 0.0f;

  const long long nchunks = p1 > p0 ? (p1 - p0 + C::BK - 1) / C::BK : 0;
  if (nchunks > 0) {
    load_chunk(0);
    cp_commit();
  }
  for (long long kc = 0; kc < nchunks; ++kc) {
    const int st = (int)(kc & 1);
    if (kc + 1 < nchunks) {
      advance();
      load_chunk(st ^ 1);
    }
    cp_commit();
    cp_wait<1>();
    __syncthreads();
    if (active) {
#pragma unroll
      for (int ks = 0; ks < C::BK / 16; ++ks) {
        uint32_t af[C::MT][4], bfr[C::NT][2];
        const int j = lane >> 3, r8 = lane & 7;
#pragma unroll
        for (int mt = 0; mt < C::MT; ++mt) {
          // A = dz^T: rows k (pixels) of [pixel][co], transposed by ldmatrix
          const int k = ks * 16 + r8 + (j >= 2 ? 8 : 0);
          const int m = wm * C::TM + mt * 16 + ((j & 1) ? 8 : 0);
          ldsm_x4_t(af[mt], &As[st][k * C::LDA + m]);
        }
#pragma unroll
        for (int nt = 0; nt < C::NT; ++nt) {
          const int k = ks * 16 + r8 + ((j & 1) ? 8 : 0);
          const int n = wn * C::TN + nt * 8;
          ldsm_x2_t(bfr[nt], &Bs[st][k * C::LDB + n]);
        }
#pragma unroll
        for (int mt = 0; mt < C::MT; ++mt)
#pragma unroll
          for (int nt = 0; nt < C::NT; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt]);
      }
    }
    __syncthreads();
  }
  if (!active) return;
  // partial[split][co][tap][ci]
  const int g = lane >> 2, t = lane & 3;
  float* out = partial + (size_t)split * Cout * 9 * Cin;
#pragma unroll
  for (int mt = 0; mt < C::MT; ++mt)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int co = co0 + wm * C::TM + mt * 16 + g + half * 8;
#pragma unroll
      for (int nt = 0; nt < C::NT; ++nt) {
        const int ci = ci0 + wn * C::TN + nt * 8 + 2 * t;
        float* o = out + ((size_t)co * 9 + tap) * Cin + ci;
        o[0] = acc[mt][nt][half * 2 + 0];
        o[1] = acc[mt][nt][half * 2 + 1];
      }
    }
}

__global__ void k_sum_partials(const float* __restrict__ partial, int splits, size_t n, float* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int k = 0; k < splits; ++k) s += partial[(size_t)k * n + i];
  out[i] = s;
}

template <int BM, int BN>
void launch_wgrad(const bf16* x, const bf16* dz, int N, int H, int W, int Cin, int Cout, int splits, long long chunk,
                  float* partial, cudaStream_t s) {
  dim3 grid((unsigned)(Cout / BM), (unsigned)(Cin / BN), (unsigned)(9 * splits));
  k_wgrad<BM, BN><<<grid, kThreads, 0, s>>>(x, dz, N, H, W, Cin, Cout, splits, chunk, partial);
}

template <int BM>
void wgrad_bm(const bf16* x, const bf16* dz, int N, int H, int W, int Cin, int Cout, int splits, long long chunk,
              float* partial, cudaStream_t s) {
  if (Cin % 64 == 0) launch_wgrad<BM, 64>(x, dz, N, H, W, Cin, Cout, splits, chunk, partial, s);
  else if (Cin % 32 == 0) launch_wgrad<BM, 32>(x, dz, N, H, W, Cin, Cout, splits, chunk, partial, s);
  else launch_wgrad<BM, 16>(x, dz, N, H, W, Cin, Cout, splits, chunk, partial, s);
}

int tile_m(int Cout) { return Cout % 64 == 0 ? 64 : (Cout % 32 == 0 ? 32 : 16); }
int tile_n(int Cin) { return Cin % 64 == 0 ? 64 : (Cin % 32 == 0 ? 32 : 16); }

int auto_splits(long long M, int Cin, int Cout) {
  const long long tiles = (long long)(Cout / tile_m(Cout)) * (Cin / tile_n(Cin)) * 9;
  long long s = (8 * 152 + tiles - 1) / tiles;                 // enough CTAs to fill every SM several times
  const long long max_s = (M + 1023) / 1024;                  // at least 1024 pixels per split
  if (s > max_s) s = max_s;
  if (s < 1) s = 1;
  return (int)s;
}

// ---------------------------------------------------------------------------
// elementwise and reductions
// ---------------------------------------------------------------------------
constexpr int kEw = 256;
inline unsigned ew_blocks(size_t n) { return (unsigned)((n + kEw - 1) / kEw); }

__global__ void k_flip(const bf16* __restrict__ w, int Cin, int Cout, bf16* __restrict__ wt) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t n = (size_t)Cout * 9 * Cin;
  if (i >= n) return;
  const int ci = (int)(i % Cin), tap = (int)((i / Cin) % 9), co = (int)(i / ((size_t)9 * Cin));
  const int ky = tap / 3, kx = tap % 3;
  wt[((size_t)ci * 9 + (2 - ky) * 3 + (2 - kx)) * Cout + co] = w[i];
}

// 8 bfloat16 values <-> 8 floats
struct V8 {
  float v[8];
};
__device__ __forceinline__ V8 ld8(const bf16* p) {
  const uint4 u = *reinterpret_cast<const uint4*>(p);
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
  V8 r;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float2 f = __bfloat1622float2(h[k]);
    r.v[2 * k] = f.x;
    r.v[2 * k + 1] = f.y;
  }
  return r;
}
__device__ __forceinline__ void st8(bf16* p, const V8& r) {
  uint4 u;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
  for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(r.v[2 * k], r.v[2 * k + 1]);
  *reinterpret_cast<uint4*>(p) = u;
}

__global__ void k_gelu_bwd(const bf16* __restrict__ dy, const bf16* __restrict__ z, size_t n8, bf16* __restrict__ dz) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n8) return;
  V8 a = ld8(dy + 8 * i);
  const V8 b = ld8(z + 8 * i);
#pragma unroll
  for (int k = 0; k < 8; ++k) a.v[k] *= gelu_grad_f(b.v[k]);
  st8(dz + 8 * i, a);
}

constexpr int kBiasBlocks = 512;
constexpr int kBiasThreads = 256;

// Per-block channel sums of dz over a pixel range: each thread owns 8
// channels of every (kBiasThreads / (C/8))-th pixel, then the block adds its
// rows in a fixed order.  C % 8 == 0, C <= 8 * kBiasThreads.
__global__ void __launch_bounds__(kBiasThreads) k_bias_partial(const bf16* __restrict__ dz, size_t P, int C,
                                                               float* __restrict__ partial) {
  __shared__ float s[kBiasThreads * 8];
  const int vpp = C / 8, ppi = kBiasThreads / vpp;
  const int lv = threadIdx.x % vpp, lp = threadIdx.x / vpp;
  float acc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  if (lp < ppi) {
    const size_t per = (P + gridDim.x - 1) / gridDim.x;
    const size_t lo = (size_t)blockIdx.x * per, hi = min(P, lo + per);
    for (size_t p = lo + lp; p < hi; p += ppi) {
      const V8 v = ld8(dz + p * C + 8 * lv);
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[k] += v.v[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) s[threadIdx.x * 8 + k] = acc[k];
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    const int v = c / 8, k = c % 8;
    float t = 0.0f;
    for (int q = 0; q < ppi; ++q) t += s[(q * vpp + v) * 8 + k];
    partial[(size_t)blockIdx.x * C + c] = t;
  }
}

// 8 channels per thread: i indexes (output pixel, channel group)
__global__ void k_pool2(const bf16* __restrict__ x, int N, int H, int W, int C, bf16* __restrict__ y) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int h = H / 2, w = W / 2, cg = C / 8;
  const size_t n_out = (size_t)N * h * w * cg;
  if (i >= n_out) return;
  const int c = (int)(i % cg) * 8;
  const size_t pix = i / cg;
  const int xo = (int)(pix % w), yo = (int)((pix / w) % h), n = (int)(pix / ((size_t)w * h));
  const size_t b = (((size_t)n * H + 2 * yo) * W + 2 * xo) * C + c;
  const V8 a = ld8(x + b), bb = ld8(x + b + C), cc = ld8(x + b + (size_t)W * C), d = ld8(x + b + (size_t)W * C + C);
  V8 r;
#pragma unroll
  for (int k = 0; k < 8; ++k) r.v[k] = 0.25f * ((a.v[k] + bb.v[k]) + (cc.v[k] + d.v[k]));
  st8(y + pix * C + c, r);
}

__global__ void k_pool2_bwd(const bf16* __restrict__ dy, int N, int H, int W, int C, bf16* __restrict__ dx) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int cg = C / 8;
  const size_t n_in = (size_t)N * H * W * cg;
  if (i >= n_in) return;
  const int c = (int)(i % cg) * 8;
  const size_t pix = i / cg;
  const int xx = (int)(pix % W), yy = (int)((pix / W) % H), n = (int)(pix / ((size_t)W * H));
  V8 r = ld8(dy + (((size_t)n * (H / 2) + yy / 2) * (W / 2) + xx / 2) * C + c);
#pragma unroll
  for (int k = 0; k < 8; ++k) r.v[k] *= 0.25f;
  st8(dx + pix * C + c, r);
}

__global__ void k_up2(const bf16* __restrict__ x, int N, int h, int w, int C, bf16* __restrict__ y, int Cy, int coff) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int cg = C / 8;
  const size_t n_out = (size_t)N * 2 * h * 2 * w * cg;
  if (i >= n_out) return;
  const int c = (int)(i % cg) * 8;
  const size_t pix = i / cg;
  const int W = 2 * w, H = 2 * h;
  const int xx = (int)(pix % W), yy = (int)((pix / W) % H), n = (int)(pix / ((size_t)W * H));
  *reinterpret_cast<uint4*>(y + pix * Cy + coff + c) =
      *reinterpret_cast<const uint4*>(x + (((size_t)n * h + yy / 2) * w + xx / 2) * C + c);
}

__global__ void k_up2_bwd(const bf16* __restrict__ dy, int N, int h, int w, int Cy, int coff, int C,
                          bf16* __restrict__ dx) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int cg = C / 8;
  const size_t n_in = (size_t)N * h * w * cg;
  if (i >= n_in) return;
  const int c = (int)(i % cg) * 8;
  const size_t pix = i / cg;
  const int xo = (int)(pix % w), yo = (int)((pix / w) % h), n = (int)(pix / ((size_t)w * h));
  const int W = 2 * w;
  const size_t b = (((size_t)n * 2 * h + 2 * yo) * W + 2 * xo) * Cy + coff + c;
  const V8 a = ld8(dy + b), bb = ld8(dy + b + Cy), cc = ld8(dy + b + (size_t)W * Cy),
           d = ld8(dy + b + (size_t)W * Cy + Cy);
  V8 r;
#pragma unroll
  for (int k = 0; k < 8; ++k) r.v[k] = (a.v[k] + bb.v[k]) + (cc.v[k] + d.v[k]);
  st8(dx + pix * C + c, r);
}

__global__ void k_copy_ch(const bf16* __restrict__ src, size_t P, int Cs, bf16* __restrict__ dst, int Cd, int coff) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int cg = Cs / 8;
  if (i >= P * cg) return;
  const size_t p = i / cg;
  const int c = (int)(i % cg) * 8;
  *reinterpret_cast<uint4*>(dst + p * Cd + coff + c) = *reinterpret_cast<const uint4*>(src + p * Cs + c);
}

__global__ void k_add_ch(const bf16* __restrict__ src, size_t P, int Cs, int coff, int C, bf16* __restrict__ dst) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int cg = C / 8;
  if (i >= P * cg) return;
  const size_t p = i / cg;
  const int c = (int)(i % cg) * 8;
  V8 a = ld8(dst + p * C + c);
  const V8 b = ld8(src + p * Cs + coff + c);
#pragma unroll
  for (int k = 0; k < 8; ++k) a.v[k] += b.v[k];
  st8(dst + p * C + c, a);
}

constexpr int kLossBlocks = 512;

__global__ void k_masked_mse(const bf16* __restrict__ x, const bf16* __restrict__ out, const bf16* __restrict__ xn,
                             size_t P, int C, bf16* __restrict__ dout, float* __restrict__ partial, float inv_count) {
  __shared__ float s_e[kEw], s_n[kEw];
  float e = 0.0f, nf = 0.0f;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
    const size_t b = p * C;
    const bool fluid = __bfloat162float(x[b + 3]) == 0.0f;
    for (int c = 0; c < C; ++c) {
      float g = 0.0f;
      if (c < 3 && fluid) {
        const float d = (__bfloat162float(x[b + c]) + __bfloat162float(out[b + c])) - __bfloat162float(xn[b + c]);
        e += d * d;
        g = 2.0f * d * inv_count;
      }
      dout[b + c] = __float2bfloat16_rn(g);
    }
    nf += fluid ? 1.0f : 0.0f;
  }
  s_e[threadIdx.x] = e;
  s_n[threadIdx.x] = nf;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s_e[threadIdx.x] += s_e[threadIdx.x + w];
      s_n[threadIdx.x] += s_n[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = s_e[0];
    partial[2 * blockIdx.x + 1] = s_n[0];
  }
}

__global__ void k_adamw(float* __restrict__ w, bf16* __restrict__ w16, const float* __restrict__ g,
                        float* __restrict__ m, float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps,
                        float wd, float c1, float c2) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = fmaf(b1, m[i], (1.0f - b1) * gi);
  const float vi = fmaf(b2, v[i], (1.0f - b2) * gi * gi);
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * ((mi * c1) / (sqrtf(vi * c2) + eps) + wd * w[i]);
  w[i] = wi;
  if (w16) w16[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(const float* __restrict__ src, size_t n, bf16* __restrict__ dst) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

}  // namespace
}  // namespace sg

using namespace sg;
using fd::as_stream;
using fd::check_launch;

extern "C" {

int sg_conv3x3(const void* x, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout, int act,
               void* z, void* y, void* stream) {
  FD_REQUIRE(x && w && (z || y) && N > 0 && H > 0 && W > 0, FD_ERR_ARG, "sg_conv3x3: bad arguments");
  FD_REQUIRE(Cin % 16 == 0 && Cout % 16 == 0 && Cin > 0 && Cout > 0, FD_ERR_SHAPE,
             "sg_conv3x3: channel counts must be positive multiples of 16 (got %d -> %d)", Cin, Cout);
  FD_REQUIRE(act == SG_ACT_NONE || act == SG_ACT_GELU, FD_ERR_ARG, "sg_conv3x3: activation %d", act);
  FD_REQUIRE(((uintptr_t)x | (uintptr_t)w) % 16 == 0, FD_ERR_ARG, "sg_conv3x3: x and w must be 16-byte aligned");
  cudaStream_t s = as_stream(stream);
  const bf16 *xb = (const bf16*)x, *wb = (const bf16*)w;
  if (Cin % 64 == 0) conv_bk<64>(xb, N, H, W, Cin, wb, bias, Cout, act, (bf16*)z, (bf16*)y, s);
  else if (Cin % 32 == 0) conv_bk<32>(xb, N, H, W, Cin, wb, bias, Cout, act, (bf16*)z, (bf16*)y, s);
  else conv_bk<16>(xb, N, H, W, Cin, wb, bias, Cout, act, (bf16*)z, (bf16*)y, s);
  return check_launch("sg_conv3x3");
}

int sg_flip_weights(const void* w, int Cin, int Cout, void* wt, void* stream) {
  FD_REQUIRE(w && wt && Cin > 0 && Cout > 0, FD_ERR_ARG, "sg_flip_weights: bad arguments");
  const size_t n = (size_t)Cout * 9 * Cin;
  k_flip<<<ew_blocks(n), kEw, 0, as_stream(stream)>>>((const bf16*)w, Cin, Cout, (bf16*)wt);
  return check_launch("sg_flip_weights");
}

size_t sg_wgrad_partial_floats(int N, int H, int W, int Cin, int Cout) {
  if (N <= 0 || H <= 0 || W <= 0 || Cin <= 0 || Cout <= 0) return 0;
  long long s = auto_splits((long long)N * H * W, Cin, Cout);
  if (W % 128 == 0 && Cin % 16 == 0 && Cout % 16 == 0) {
    // the tcgen05 weight gradient: the larger channel count on the MMA's 128 rows, three taps per CTA,
    // at most two waves of one CTA per SM, no more splits than chunks of 128 pixels (sg_conv3x3_wgrad_tc)
    const int mrows = Cin > Cout ? Cin : Cout, nch = Cin > Cout ? Cout : Cin;
    const int bn = nch % 128 == 0 ? 128 : (nch % 64 == 0 ? 64 : (nch % 32 == 0 ? 32 : 16));
    const long long per = (long long)((mrows + 127) / 128) * (nch / bn) * 3;
    long long t = (2 * 152) / per;
    if (t < 1) t = 1;
    const long long chunks = (long long)N * H * (W / 128);
    if (t > chunks) t = chunks;
    if (t > s) s = t;
  }
  return (size_t)s * Cout * 9 * Cin;
}

int sg_conv3x3_wgrad(const void* x, const void* dz, int N, int H, int W, int Cin, int Cout, float* dw,
                     float* partial, size_t partial_floats, int splits, void* stream) {
  FD_REQUIRE(x && dz && dw && partial && N > 0 && H > 0 && W > 0, FD_ERR_ARG, "sg_conv3x3_wgrad: bad arguments");
  FD_REQUIRE(Cin % 16 == 0 && Cout % 16 == 0 && Cin > 0 && Cout > 0, FD_ERR_SHAPE,
             "sg_conv3x3_wgrad: channel counts must be positive multiples of 16 (got %d -> %d)", Cin, Cout);
  const long long M = (long long)N * H * W;
  if (splits <= 0) splits = auto_splits(M, Cin, Cout);
  const size_t n = (size_t)Cout * 9 * Cin;
  FD_REQUIRE((size_t)splits * n <= partial_floats, FD_ERR_ARG, "sg_conv3x3_wgrad: partial buffer too small");
  long long chunk = (M + splits - 1) / splits;
  chunk = (chunk + 63) / 64 * 64;
  cudaStream_t s = as_stream(stream);
  const bf16 *xb = (const bf16*)x, *db = (const bf16*)dz;
  switch (tile_m(Cout)) {
    case 64: wgrad_bm<64>(xb, db, N, H, W, Cin, Cout, splits, chunk, partial, s); break;
    case 32: wgrad_bm<32>(xb, db, N, H, W, Cin, Cout, splits, chunk, partial, s); break;
    default: wgrad_bm<16>(xb, db, N, H, W, Cin, Cout, splits, chunk, partial, s); break;
  }
  k_sum_partials<<<ew_blocks(n), kEw, 0, s>>>(partial, splits, n, dw);
  return check_launch("sg_conv3x3_wgrad");
}

size_t sg_bias_partial_floats(int C) { return (size_t)kBiasBlocks * (C > 0 ? C : 0); }

int sg_bias_grad(const void* dz, size_t P, int C, float* db, float* partial, void* stream) {
  FD_REQUIRE(dz && db && partial && C > 0 && C % 8 == 0 && C <= 8 * kBiasThreads, FD_ERR_ARG,
             "sg_bias_grad: bad arguments");
  cudaStream_t s = as_stream(stream);
  k_bias_partial<<<kBiasBlocks, kBiasThreads, 0, s>>>((const bf16*)dz, P, C, partial);
  k_sum_partials<<<ew_blocks((size_t)C), kEw, 0, s>>>(partial, kBiasBlocks, (size_t)C, db);
  return check_launch("sg_bias_grad");
}

int sg_gelu_bwd(const void* dy, const void* z, size_t n, void* dz, void* stream) {
  FD_REQUIRE(dy && z && dz && n % 8 == 0, FD_ERR_ARG, "sg_gelu_bwd: bad arguments (n must be a multiple of 8)");
  k_gelu_bwd<<<ew_blocks(n / 8), kEw, 0, as_stream(stream)>>>((const bf16*)dy, (const bf16*)z, n / 8, (bf16*)dz);
  return check_launch("sg_gelu_bwd");
}

int sg_pool2(const void* x, int N, int H, int W, int C, void* y, void* stream) {
  FD_REQUIRE(x && y && H % 2 == 0 && W % 2 == 0 && C % 8 == 0, FD_ERR_ARG, "sg_pool2: bad arguments");
  const size_t n = (size_t)N * (H / 2) * (W / 2) * (C / 8);
  k_pool2<<<ew_blocks(n), kEw, 0, as_stream(stream)>>>((const bf16*)x, N, H, W, C, (bf16*)y);
  return check_launch("sg_pool2");
}

int sg_pool2_bwd(const void* dy, int N, int H, int W, int C, void* dx, void* stream) {
  FD_REQUIRE(dy && dx && H % 2 == 0 && W % 2 == 0 && C % 8 == 0, FD_ERR_ARG, "sg_pool2_bwd: bad arguments");
  const size_t n = (size_t)N * H * W * (C / 8);
  k_pool2_bwd<<<ew_blocks(n), kEw, 0, as_stream(stream)>>>((const bf16*)dy, N, H, W, C, (bf16*)dx);
  return check_launch("sg_pool2_bwd");
}

int sg_up2(const void* x, int N, int h, int w, int C, void* y, int Cy, int coff, void* stream) {
  FD_REQUIRE(x && y && coff >= 0 && coff + C <= Cy && C % 8 == 0 && Cy % 8 == 0 && coff % 8 == 0, FD_ERR_ARG,
             "sg_up2: bad arguments");
  const size_t n = (size_t)N * 4 * h * w * (C / 8);
  k_up2<<<ew_blocks(n), kEw, 0, as_stream(stream)>>>((const bf16*)x, N, h, w, C, (bf16*)y, Cy, coff);
  return check_launch("sg_up2");
}

int sg_up2_bwd(const void* dy, int N, int h, int w, int Cy, int coff, int C, void* dx, void* stream) {
  FD_REQUIRE(dy && dx && coff >= 0 && coff + C <= Cy && C % 8 == 0 && Cy % 8 == 0 && coff % 8 == 0, FD_ERR_ARG,
             "sg_up2_bwd: bad arguments");
  const size_t n = (size_t)N * h * w * (C / 8);
  k_up2_bwd<<<ew_blocks(n), kEw, 0, as_stream(stream)>>>((const bf16*)dy, N, h, w, Cy, coff, C, (bf16*)dx);
  return check_launch("sg_up2_bwd");
}

int sg_copy_channels(const void* src, size_t P, int Cs, void* dst, int Cd, int coff, void* stream) {
  FD_REQUIRE(src && dst && coff >= 0 && coff + Cs <= Cd && Cs % 8 == 0 && Cd % 8 == 0 && coff % 8 == 0, FD_ERR_ARG,
             "sg_copy_channels: bad arguments");
  k_copy_ch<<<ew_blocks(P * (Cs / 8)), kEw, 0, as_stream(stream)>>>((const bf16*)src, P, Cs, (bf16*)dst, Cd, coff);
  return check_launch("sg_copy_channels");
}

int sg_add_channels(const void* src, size_t P, int Cs, int coff, int C, void* dst, void* stream) {
  FD_REQUIRE(src && dst && coff >= 0 && coff + C <= Cs && C % 8 == 0 && Cs % 8 == 0 && coff % 8 == 0, FD_ERR_ARG,
             "sg_add_channels: bad arguments");
  k_add_ch<<<ew_blocks(P * (C / 8)), kEw, 0, as_stream(stream)>>>((const bf16*)src, P, Cs, coff, C, (bf16*)dst);
  return check_launch("sg_add_channels");
}

int sg_loss_blocks(void) { return kLossBlocks; }

int sg_masked_mse(const void* x, const void* out, const void* xn, size_t P, int C, void* dout, float* loss_partial,
                  float inv_count, void* stream) {
  FD_REQUIRE(x && out && xn && dout && loss_partial && C >= 4, FD_ERR_ARG, "sg_masked_mse: bad arguments");
  k_masked_mse<<<kLossBlocks, kEw, 0, as_stream(stream)>>>((const bf16*)x, (const bf16*)out, (const bf16*)xn, P, C,
                                                          (bf16*)dout, loss_partial, inv_count);
  return check_launch("sg_masked_mse");
}

int sg_adamw(float* w, void* w16, const float* g, float* m, float* v, size_t n, float lr, float beta1, float beta2,
             float eps, float weight_decay, int step, void* stream) {
  FD_REQUIRE(w && g && m && v && step >= 1, FD_ERR_ARG, "sg_adamw: bad arguments");
  const float c1 = 1.0f / (1.0f - powf(beta1, (float)step));
  const float c2 = 1.0f / (1.0f - powf(beta2, (float)step));
  k_adamw<<<ew_blocks(n), kEw, 0, as_stream(stream)>>>(w, (bf16*)w16, g, m, v, n, lr, beta1, beta2, eps,
                                                       weight_decay, c1, c2);
  return check_launch("sg_adamw");
}

int sg_to_bf16(const float* src, size_t n, void* dst, void* stream) {
  FD_REQUIRE(src && dst, FD_ERR_ARG, "sg_to_bf16: NULL pointer");
  k_to_bf16<<<ew_blocks(n), kEw, 0, as_stream(stream)>>>(src, n, (bf16*)dst);
  return check_launch("sg_to_bf16");
}

}  // extern "C"
