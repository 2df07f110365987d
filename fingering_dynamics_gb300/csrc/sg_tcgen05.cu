// 3x3 convolution (forward and data gradient) of the learned surrogate on the
// fifth-generation tensor cores: tcgen05.mma with bfloat16 operands read from
// shared memory through matrix descriptors and the FP32 accumulator in tensor
// memory (TMEM).
//
// Implicit GEMM, M = pixels, N = output channels, K = 9 x input channels.  A
// CTA of 128 threads owns 128 pixels x BN channels; the accumulator is 128
// TMEM lanes x BN columns.  K advances in chunks of BK input channels of one
// tap (the nine taps of a channel chunk back to back): all threads copy the
// chunk's A (im2col rows) and B (weights) tiles into shared memory with
// cp.async, in the canonical K-major layout without swizzle (core matrices
// of 8 rows x 16 bytes; LBO = 128 B between the two core matrices of a K=16
// slice, SBO = BK/8 x 128 B between 8-row groups), make them visible to the
// async proxy, and one thread issues BK/16 MMAs (M=128, N=BN, K=16) and
// commits them to the stage's mbarrier.  Four stages: three chunks are in
// flight while one is multiplied, and a stage is refilled once the MMAs that
// read it have completed.  The epilogue reads the accumulator
// with tcgen05.ld (each warp its 32 lanes = 32 pixels), adds the bias,
// applies GELU and stores bfloat16.
//
// The TMA-fed variant (k_conv3x3_tma, sg_conv3x3_tma) keeps the halo tiles'
// shared-memory layout but fills it with tensor-map boxes issued by one
// thread into a ring of stages completing on mbarriers (zero fill outside
// the image is the convolution's padding), and the same thread issues the
// MMAs as soon as a stage has landed: no thread copies operands and no CTA
// barrier separates the chunks.
//
// Every mbarrier wait is bounded; a wait that gives up sets bit 0 of
// g_sg_tc_error (read by sg_tc_status) and the kernel continues without
// hanging; TMEM is always released.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/fdsurrogate.h"
#include "fd_host.h"
#include "fd_tmap.h"

namespace sg {

__device__ unsigned int g_sg_tc_error = 0;

namespace {

using bf16 = __nv_bfloat16;
constexpr int kTcThreads = 128;
constexpr int kTcBM = 128;
constexpr unsigned kTcWaitLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp16_l1(void* dst, const void* src, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}

// bounded wait for phase `parity` of an mbarrier
__device__ __forceinline__ void mbar_wait(uint64_t* bar, unsigned parity) {
  const uint32_t a = smem_u32(bar);
  for (unsigned it = 0; it < kTcWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return;
  }
  atomicOr(&g_sg_tc_error, 1u);
}

// bounded wait that reports whether the phase completed.  `bail`: also give
// up once any wait of the launch has given up (the error word is set), so a
// failure common to every CTA does not cost every CTA a wait's full limit;
// the waits that drain copies and MMAs in flight before a CTA exits keep the
// full limit.
__device__ __forceinline__ bool mbar_wait_ok(uint64_t* bar, unsigned parity, bool bail) {
  const uint32_t a = smem_u32(bar);
  for (unsigned it = 0; it < kTcWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (bail && (it & 1023u) == 1023u && *reinterpret_cast<volatile unsigned*>(&g_sg_tc_error) != 0u) return false;
  }
  atomicOr(&g_sg_tc_error, 1u);
  return false;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// one box of a 3-D / 4-D tensor map into shared memory (128-byte aligned
// destination; the innermost coordinate times the element size a multiple of
// 16 bytes)
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// shared-memory matrix descriptor: canonical K-major layout, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of this architecture
  return d;                // base offset 0, layout "no swizzle" (bits 61..63 = 0)
}

// instruction descriptor of kind::f16: D FP32, A and B bfloat16, both K-major
template <int M, int N>
__device__ __forceinline__ constexpr uint32_t instr_desc() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ float gelu_f(float z) {
  const float u = 0.7978845608028654f * fmaf(0.044715f * z * z, z, z);
  return 0.5f * z * (1.0f + tanhf(u));
}

// 32 lanes x 16 columns of 32-bit accumulators: thread t gets lane base+t, columns col..col+15
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

constexpr int kTcStages = 4;

template <int BN, int BK>
struct TcCfg {
  static constexpr int S = kTcStages;
  static constexpr int A_BYTES = kTcBM * BK * 2;  // 128 rows x BK bfloat16
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int SBO = (BK / 8) * 128;       // bytes between 8-row groups
  static constexpr int LBO = 128;                  // bytes between the K=0..7 and K=8..15 core matrices
  static constexpr int SMEM = S * STAGE + 128;     // stages + barriers + TMEM address
  static constexpr int COLS = BN < 32 ? 32 : BN;   // TMEM columns (power of two >= 32)
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "N of an M=128 MMA");
  static_assert(BK % 16 == 0, "K chunk");
};

// byte offset of element (row, k) in a canonical K-major tile
template <int BK>
__device__ __forceinline__ uint32_t tile_off(int row, int k) {
  return (uint32_t)((row & 7) * 16 + (row >> 3) * ((BK / 8) * 128) + (k >> 3) * 128 + (k & 7) * 2);
}

template <int BN, int BK>
__global__ void __launch_bounds__(kTcThreads) k_conv3x3_tc(const bf16* __restrict__ x, int N, int H, int W,
                                                          int Cin, const bf16* __restrict__ w,
                                                          const float* __restrict__ bias, int Cout, int act,
                                                          bf16* __restrict__ z, bf16* __restrict__ y) {
  using C = TcCfg<BN, BK>;
  extern __shared__ __align__(1024) char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + C::S * C::STAGE);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + C::S * C::STAGE + 8 * C::S);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long M = (long long)N * H * W;
  const long long m0 = (long long)blockIdx.x * kTcBM;
  const int co0 = blockIdx.y * BN;
  const int nk = 9 * (Cin / BK);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(C::COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < C::S; ++i) mbar_init(&bars[i]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // this thread's A rows: pixel bases at the centre tap and tap-validity masks
  constexpr int VPR = BK / 8;
  constexpr int A_PER = kTcBM * VPR / kTcThreads;
  static_assert(A_PER * kTcThreads == kTcBM * VPR, "A vectors per thread");
  const bf16* a_base[A_PER];
  uint32_t a_valid[A_PER], a_soff[A_PER];
#pragma unroll
  for (int i = 0; i < A_PER; ++i) {
    const int v = tid + i * kTcThreads;
    const int row = v / VPR, kv = v % VPR;
    const long long p = m0 + row;
    a_soff[i] = tile_off<BK>(row, kv * 8);
    a_base[i] = x;
    a_valid[i] = 0u;
    if (p < M) {
      const int rem = (int)(p % ((long long)H * W));
      const int yy = rem / W, xx = rem % W;
      a_base[i] = x + p * Cin + kv * 8;
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int ty = yy + t / 3 - 1, tx = xx + t % 3 - 1;
        if (ty >= 0 && ty < H && tx >= 0 && tx < W) a_valid[i] |= 1u << t;
      }
    }
  }

  auto load_chunk = [&](int kc, int st) {
    char* As = smem + st * C::STAGE;
    char* Bs = As + C::A_BYTES;
    const int tap = kc % 9, ci0 = (kc / 9) * BK;
    const long long toff = ((long long)(tap / 3 - 1) * W + (tap % 3 - 1)) * Cin + ci0;
#pragma unroll
    for (int i = 0; i < A_PER; ++i) {
      const bool ok = (a_valid[i] >> tap) & 1u;
      cp16_l1(As + a_soff[i], ok ? a_base[i] + toff : x, ok ? 16 : 0);
    }
    for (int v = tid; v < BN * VPR; v += kTcThreads) {
      const int r = v / VPR, kv = v % VPR;
      cp16(Bs + tile_off<BK>(r, kv * 8), w + ((long long)(co0 + r) * 9 + tap) * Cin + ci0 + kv * 8);
    }
  };

  constexpr uint32_t idesc = instr_desc<kTcBM, BN>();
  unsigned phase = 0;  // bit s: parity of the next completion of stage s
  auto wait_stage = [&](int s) {
    mbar_wait(&bars[s], (phase >> s) & 1u);
    phase ^= 1u << s;
  };
  // prologue: chunks 0 .. S-2 in flight
#pragma unroll
  for (int i = 0; i < C::S - 1; ++i) {
    if (i < nk) load_chunk(i, i);
    cp_commit();
  }
  for (int kc = 0; kc < nk; ++kc) {
    const int st = kc % C::S;
    const int nxt = kc + C::S - 1;  // refills the stage chunk kc-1 used
    if (nxt < nk) {
      if (kc >= 1) wait_stage((kc - 1) % C::S);
      load_chunk(nxt, nxt % C::S);
    }
    cp_commit();
    cp_wait<C::S - 1>();  // chunk kc has landed
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // cp.async data -> tensor core reads
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(smem + st * C::STAGE), b0 = a0 + C::A_BYTES;
#pragma unroll
      for (int s = 0; s < BK / 16; ++s) {
        const uint64_t ad = smem_desc(a0 + s * 2 * C::LBO, C::LBO, C::SBO);
        const uint64_t bd = smem_desc(b0 + s * 2 * C::LBO, C::LBO, C::SBO);
        tc_mma(tmem, ad, bd, idesc, (kc > 0 || s > 0) ? 1u : 0u);
      }
      tc_commit(&bars[st]);
    }
  }
  // the commits not waited for in the loop: chunks max(0, nk-S) .. nk-1
  for (int c = (nk > C::S ? nk - C::S : 0); c < nk; ++c) wait_stage(c % C::S);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // epilogue: warp w holds pixels m0 + 32 w + lane
  const long long p = m0 + warp * 32 + lane;
#pragma unroll
  for (int c0 = 0; c0 < BN; c0 += 16) {
    float v[16];
    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
    if (p < M) {
      const int co = co0 + c0;
      uint32_t zw[8], yw[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        float t0 = v[2 * i] + (bias ? bias[co + 2 * i] : 0.0f);
        float t1 = v[2 * i + 1] + (bias ? bias[co + 2 * i + 1] : 0.0f);
        const __nv_bfloat162 zp = __floats2bfloat162_rn(t0, t1);
        zw[i] = *reinterpret_cast<const uint32_t*>(&zp);
        if (act == SG_ACT_GELU) {
          t0 = gelu_f(t0);
          t1 = gelu_f(t1);
        }
        const __nv_bfloat162 yp = __floats2bfloat162_rn(t0, t1);
        yw[i] = *reinterpret_cast<const uint32_t*>(&yp);
      }
      const size_t o = (size_t)p * Cout + co;
      if (z) {
        reinterpret_cast<uint4*>(z + o)[0] = make_uint4(zw[0], zw[1], zw[2], zw[3]);
        reinterpret_cast<uint4*>(z + o)[1] = make_uint4(zw[4], zw[5], zw[6], zw[7]);
      }
      if (y) {
        reinterpret_cast<uint4*>(y + o)[0] = make_uint4(yw[0], yw[1], yw[2], yw[3]);
        reinterpret_cast<uint4*>(y + o)[1] = make_uint4(yw[4], yw[5], yw[6], yw[7]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Halo-tile variant for images whose width is a multiple of 128: a CTA owns
// 128 pixels of one image row.  Per input-channel chunk it copies the three
// input rows y-1, y, y+1 over 130 pixels (x0-1 .. x0+128, zeros outside the
// image) once, and the weights of all nine taps; each tap's A operand is the
// 128-row window that starts (1 + kx) pixels into row block ky + 1.  The
// window can start on any pixel because the rows of a block are 16 bytes
// apart with no gap between 8-row groups (SBO = 128 B) and the two K halves
// of a 16-wide slice sit a whole block column apart (LBO = 130 x 16 B).  The
// input is read once per tile instead of nine times.
// ---------------------------------------------------------------------------
constexpr int kHaloPx = kTcBM + 2;

template <int BN, int BK, int R>
struct HaloCfg {
  static constexpr int LBO_A = kHaloPx * 16;            // between the K-slices of a row block
  static constexpr int BLK = (BK / 8) * LBO_A;          // one input row block
  static constexpr int A_BYTES = (R + 2) * BLK;         // input rows y0-1 .. y0+R
  static constexpr int TB = BN * BK * 2;                // one tap's weights (canonical K-major)
  static constexpr int B_BYTES = 9 * TB;
  static constexpr int STAGE = (A_BYTES + B_BYTES + 127) / 128 * 128;
  static constexpr int SMEM = 2 * STAGE + 128;
  static constexpr int NCOL = R * BN;                   // R accumulators of BN columns
  static constexpr int COLS = NCOL <= 32 ? 32 : (NCOL <= 64 ? 64 : (NCOL <= 128 ? 128 : (NCOL <= 256 ? 256 : 512)));
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256 && BK % 16 == 0 && NCOL <= 512, "tile");
};

template <int BN, int BK, int R>
__global__ void __launch_bounds__(kTcThreads) k_conv3x3_tch(const bf16* __restrict__ x, int N, int H, int W,
                                                           int Cin, const bf16* __restrict__ w,
                                                           const float* __restrict__ bias, int Cout, int act,
                                                           bf16* __restrict__ z, bf16* __restrict__ y) {
  using C = HaloCfg<BN, BK, R>;
  extern __shared__ __align__(1024) char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + 2 * C::STAGE);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 2 * C::STAGE + 32);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_x = W / kTcBM;
  const int tx = blockIdx.x % tiles_x, rblk = blockIdx.x / tiles_x;  // block of R image rows
  const int row = rblk * R;                                          // first row = n * H + yy (H % R == 0)
  const int yy = row % H;
  const int x0 = tx * kTcBM;
  const int co0 = blockIdx.y * BN;
  const int nk = Cin / BK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(C::COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&bars[0]);
    mbar_init(&bars[1]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  constexpr int VPR = BK / 8;  // 16-byte vectors per pixel of a chunk
  auto load_chunk = [&](int kc, int st) {
    char* As = smem + st * C::STAGE;
    char* Bs = As + C::A_BYTES;
    const int ci0 = kc * BK;
    for (int v = tid; v < (R + 2) * kHaloPx * VPR; v += kTcThreads) {
      const int kv = v % VPR, px = (v / VPR) % kHaloPx, rb = v / (VPR * kHaloPx);
      const int sy = yy + rb - 1, sx = x0 + px - 1;
      const bool ok = sy >= 0 && sy < H && sx >= 0 && sx < W;
      const bf16* src = ok ? x + ((long long)(row + rb - 1) * W + sx) * Cin + ci0 + kv * 8 : x;
      cp16_l1(As + rb * C::BLK + kv * C::LBO_A + px * 16, src, ok ? 16 : 0);
    }
    for (int v = tid; v < 9 * BN * VPR; v += kTcThreads) {
      const int kv = v % VPR, r = (v / VPR) % BN, tap = v / (VPR * BN);
      cp16(Bs + tap * C::TB + tile_off<BK>(r, kv * 8), w + ((long long)(co0 + r) * 9 + tap) * Cin + ci0 + kv * 8);
    }
  };

  constexpr uint32_t idesc = instr_desc<kTcBM, BN>();
  unsigned phase = 0;
  auto wait_stage = [&](int s) {
    mbar_wait(&bars[s], (phase >> s) & 1u);
    phase ^= 1u << s;
  };
  load_chunk(0, 0);
  cp_commit();
  for (int kc = 0; kc < nk; ++kc) {
    const int st = kc & 1;
    if (kc + 1 < nk) {
      if (kc >= 1) wait_stage(st ^ 1);  // stage st^1 was read by the MMAs of chunk kc-1
      load_chunk(kc + 1, st ^ 1);
    }
    cp_commit();
    cp_wait<1>();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(smem + st * C::STAGE), b0 = a0 + C::A_BYTES;
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        const int ky = tap / 3, kx = tap % 3;  // row block r + ky, window start kx (= 1 + (kx - 1))
#pragma unroll
        for (int s = 0; s < BK / 16; ++s) {
          const uint64_t bd = smem_desc(b0 + tap * C::TB + s * 256, 128, (BK / 8) * 128);
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const uint64_t ad = smem_desc(a0 + (r + ky) * C::BLK + 2 * s * C::LBO_A + kx * 16, C::LBO_A, 128);
            tc_mma(tmem + (uint32_t)(r * BN), ad, bd, idesc, (kc > 0 || tap > 0 || s > 0) ? 1u : 0u);
          }
        }
      }
      tc_commit(&bars[st]);
    }
  }
  for (int c = (nk > 2 ? nk - 2 : 0); c < nk; ++c) wait_stage(c & 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

#pragma unroll 1
  for (int r = 0; r < R; ++r) {
    const long long p = ((long long)(row + r) * W + x0) + warp * 32 + lane;
#pragma unroll
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(r * BN + c0), v);
      const int co = co0 + c0;
      uint32_t zw[8], yw[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        float t0 = v[2 * i] + (bias ? bias[co + 2 * i] : 0.0f);
        float t1 = v[2 * i + 1] + (bias ? bias[co + 2 * i + 1] : 0.0f);
        const __nv_bfloat162 zp = __floats2bfloat162_rn(t0, t1);
        zw[i] = *reinterpret_cast<const uint32_t*>(&zp);
        if (act == SG_ACT_GELU) {
          t0 = gelu_f(t0);
          t1 = gelu_f(t1);
        }
        const __nv_bfloat162 yp = __floats2bfloat162_rn(t0, t1);
        yw[i] = *reinterpret_cast<const uint32_t*>(&yp);
      }
      const size_t o = (size_t)p * Cout + co;
      if (z) {
        reinterpret_cast<uint4*>(z + o)[0] = make_uint4(zw[0], zw[1], zw[2], zw[3]);
        reinterpret_cast<uint4*>(z + o)[1] = make_uint4(zw[4], zw[5], zw[6], zw[7]);
      }
      if (y) {
        reinterpret_cast<uint4*>(y + o)[0] = make_uint4(yw[0], yw[1], yw[2], yw[3]);
        reinterpret_cast<uint4*>(y + o)[1] = make_uint4(yw[4], yw[5], yw[6], yw[7]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// TMA-fed halo tiles.  A CTA owns R image rows x 128 pixels x BN output
// channels (R accumulators of BN TMEM columns); K advances in chunks of 16
// input channels, each chunk one stage of the ring:
//   A: two boxes (8 channels x 130 pixels x R+2 rows of one image) of the 4-D
//      map (C, W, H, N) over x, landing as [row][pixel][8 channels] = the
//      halo kernel's row blocks (16 B per pixel, SBO 128 B), the second
//      K-slice SLICE bytes after the first (LBO); out-of-image pixels and rows
//      read as zero, the convolution's padding;
//   B: one box (8 channels x 1 tap x BN output channels) of the 3-D map
//      (Cin, 9, Cout) over the weights per tap and K-slice, landing as BN rows
//      of 16 B (SBO 128 B), the second K-slice BN x 16 B after the first (LBO).
// Thread 0 issues the boxes of S chunks ahead, waits for a stage to land,
// issues its 9 x R MMAs and commits them to the stage's second mbarrier; the
// stage of the previous chunk is refilled once its MMAs have completed, so
// the MMAs of a chunk are queued while that wait runs.  The other threads
// wait at the CTA barrier before the epilogue.
// ---------------------------------------------------------------------------
struct ConvMaps {
  CUtensorMap x, w;
};

template <int BN, int R>
struct TmaStage {
  static constexpr int A_BOX = (R + 2) * kHaloPx * 16;      // bytes of one A box
  static constexpr int SLICE = (A_BOX + 127) / 128 * 128;   // one 8-channel slice of the halo
  static constexpr int ROWB = kHaloPx * 16;                 // one input row of a slice
  static constexpr int A_BYTES = 2 * SLICE;
  static constexpr int BSL = BN * 16;                       // one tap's K-slice of weights
  static constexpr int TB = 2 * BSL;                        // one tap's weights
  static constexpr int STAGE = A_BYTES + 9 * TB;
  static constexpr int TX = 2 * A_BOX + 18 * BSL;           // bytes the boxes of a stage bring
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "tile");
  static_assert(STAGE % 128 == 0 && SLICE % 128 == 0 && BSL % 128 == 0, "128-byte aligned box destinations");
};

template <int BN, int R, int S>
struct TmaConvCfg : TmaStage<BN, R> {
  static constexpr int OFF_BAR = S * TmaStage<BN, R>::STAGE;
  static constexpr int SMEM = OFF_BAR + 2 * S * 8 + 16 + 128;  // + mbarriers, TMEM address, alignment
  static constexpr int NCOL = R * BN;
  static constexpr int COLS = NCOL <= 32 ? 32 : (NCOL <= 64 ? 64 : (NCOL <= 128 ? 128 : (NCOL <= 256 ? 256 : 512)));
  static_assert(NCOL <= 512, "tile");
};

// shared memory of TmaConvCfg<BN, R, S> (the stage count that fits is chosen
// before the configuration is instantiated)
constexpr int tma_conv_smem(int BN, int R, int S) {
  return S * (2 * (((R + 2) * kHaloPx * 16 + 127) / 128 * 128) + 18 * BN * 16) + 2 * S * 8 + 16 + 128;
}

template <int BN, int R, int S>
__global__ void __launch_bounds__(kTcThreads, 1) k_conv3x3_tma(const __grid_constant__ ConvMaps maps, int H,
                                                              int W, int Cin, const float* __restrict__ bias,
                                                              int Cout, int act, bf16* __restrict__ z,
                                                              bf16* __restrict__ y) {
  using C = TmaConvCfg<BN, R, S>;
  extern __shared__ char smem_raw[];
  char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
  uint64_t* empty = full + S;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(empty + S);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_x = W / kTcBM;
  const int tx = blockIdx.x % tiles_x, rblk = blockIdx.x / tiles_x;
  const int row = rblk * R;  // first output row = n * H + yy (H % R == 0)
  const int n = row / H, yy = row % H;
  const int x0 = tx * kTcBM;
  const int co0 = blockIdx.y * BN;
  const int nk = Cin / 16;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(C::COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < 2 * S; ++i) mbar_init(&full[i]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (tid == 0) {
    // chunk whose boxes / MMAs are in flight on each stage and not yet waited for (-1: none)
    int pend_full[S], pend_empty[S];
#pragma unroll
    for (int i = 0; i < S; ++i) pend_full[i] = pend_empty[i] = -1;
    auto issue = [&](int kc, int st) {
      char* As = smem + st * C::STAGE;
      char* Bs = As + C::A_BYTES;
      mbar_expect_tx(&full[st], (unsigned)C::TX);
#pragma unroll
      for (int s = 0; s < 2; ++s) tma_load_4d(As + s * C::SLICE, &maps.x, kc * 16 + 8 * s, x0 - 1, yy - 1, n, &full[st]);
#pragma unroll
      for (int tap = 0; tap < 9; ++tap)
#pragma unroll
        for (int s = 0; s < 2; ++s) tma_load_3d(Bs + tap * C::TB + s * C::BSL, &maps.w, kc * 16 + 8 * s, tap, co0, &full[st]);
      pend_full[st] = kc;
    };
    constexpr uint32_t idesc = instr_desc<kTcBM, BN>();
    bool ok = true;
    for (int c = 0; c < S && c < nk; ++c) issue(c, c);
    for (int kc = 0; kc < nk && ok; ++kc) {
      const int st = kc % S;
      ok = mbar_wait_ok(&full[st], (unsigned)(kc / S) & 1u, true);
      if (!ok) break;
      pend_full[st] = -1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(smem + st * C::STAGE), b0 = a0 + C::A_BYTES;
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        const int ky = tap / 3, kx = tap % 3;
        const uint64_t bd = smem_desc(b0 + tap * C::TB, C::BSL, 128);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const uint64_t ad = smem_desc(a0 + (r + ky) * C::ROWB + kx * 16, C::SLICE, 128);
          tc_mma(tmem + (uint32_t)(r * BN), ad, bd, idesc, (kc > 0 || tap > 0) ? 1u : 0u);
        }
      }
      tc_commit(&empty[st]);
      pend_empty[st] = kc;
      // refill the stage of chunk kc-1 once its MMAs have completed
      if (kc >= 1 && kc - 1 + S < nk) {
        const int ps = (kc - 1) % S;
        ok = mbar_wait_ok(&empty[ps], (unsigned)((kc - 1) / S) & 1u, true);
        if (!ok) break;
        pend_empty[ps] = -1;
        issue(kc - 1 + S, ps);
      }
    }
    // every box and MMA issued has completed (bounded waits) before the
    // accumulators are read, the shared memory is released or TMEM freed
#pragma unroll
    for (int i = 0; i < S; ++i) {
      if (pend_full[i] >= 0) mbar_wait_ok(&full[i], (unsigned)(pend_full[i] / S) & 1u, false);
      if (pend_empty[i] >= 0) mbar_wait_ok(&empty[i], (unsigned)(pend_empty[i] / S) & 1u, false);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

#pragma unroll 1
  for (int r = 0; r < R; ++r) {
    const long long p = ((long long)(row + r) * W + x0) + warp * 32 + lane;
#pragma unroll
    for (int c0 = 0; c0 < BN; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(r * BN + c0), v);
      const int co = co0 + c0;
      uint32_t zw[8], yw[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        float t0 = v[2 * i] + (bias ? bias[co + 2 * i] : 0.0f);
        float t1 = v[2 * i + 1] + (bias ? bias[co + 2 * i + 1] : 0.0f);
        const __nv_bfloat162 zp = __floats2bfloat162_rn(t0, t1);
        zw[i] = *reinterpret_cast<const uint32_t*>(&zp);
        if (act == SG_ACT_GELU) {
          t0 = gelu_f(t0);
          t1 = gelu_f(t1);
        }
        const __nv_bfloat162 yp = __floats2bfloat162_rn(t0, t1);
        yw[i] = *reinterpret_cast<const uint32_t*>(&yp);
      }
      const size_t o = (size_t)p * Cout + co;
      if (z) {
        reinterpret_cast<uint4*>(z + o)[0] = make_uint4(zw[0], zw[1], zw[2], zw[3]);
        reinterpret_cast<uint4*>(z + o)[1] = make_uint4(zw[4], zw[5], zw[6], zw[7]);
      }
      if (y) {
        reinterpret_cast<uint4*>(y + o)[0] = make_uint4(yw[0], yw[1], yw[2], yw[3]);
        reinterpret_cast<uint4*>(y + o)[1] = make_uint4(yw[4], yw[5], yw[6], yw[7]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::COLS) : "memory");
  }
}

// Tensor maps of one call: x as (C, W, H, N) with boxes of 8 channels x 130
// pixels x R+2 rows, the weights [co][tap][ci] as (Cin, 9, Cout) with boxes of
// 8 channels x 1 tap x BN output channels.
inline int encode_conv_maps(ConvMaps& m, const bf16* x, int N, int H, int W, int Cin, const bf16* w, int Cout,
                            int R, int BN) {
  const fd::EncodeTiledFn fn = fd::encode_tiled_fn();
  FD_REQUIRE(fn != nullptr, FD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint64_t es = 2;
  const cuuint64_t xd[4] = {(cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
  const cuuint64_t xs[3] = {Cin * es, (cuuint64_t)W * Cin * es, (cuuint64_t)H * W * Cin * es};
  const cuuint32_t xb[4] = {8u, (cuuint32_t)kHaloPx, (cuuint32_t)(R + 2), 1u};
  const cuuint32_t e4[4] = {1u, 1u, 1u, 1u};
  CUresult r = fn(&m.x, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(x), xd, xs, xb, e4,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  FD_REQUIRE(r == CUDA_SUCCESS, FD_ERR_CUDA, "sg_conv3x3_tma: input tensor map (%d)", (int)r);
  const cuuint64_t wd[3] = {(cuuint64_t)Cin, 9u, (cuuint64_t)Cout};
  const cuuint64_t ws[2] = {Cin * es, 9u * Cin * es};
  const cuuint32_t wb[3] = {8u, 1u, (cuuint32_t)BN};
  r = fn(&m.w, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16*>(w), wd, ws, wb, e4,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  FD_REQUIRE(r == CUDA_SUCCESS, FD_ERR_CUDA, "sg_conv3x3_tma: weight tensor map (%d)", (int)r);
  return FD_OK;
}

#ifndef SG_TMA_PAIR
#define SG_TMA_PAIR 1
#endif
#ifndef SG_TMA_BN_MAX  // output channels of the widest tile (128 or 64)
#define SG_TMA_BN_MAX 128
#endif
constexpr int kSmPerSmBytes = 233472;  // shared memory of an SM (228 KB), 1 KB of it reserved per CTA

template <int BN, int R, int S>
int launch_tma_r(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
                 bf16* z, bf16* y, cudaStream_t s) {
  using C = TmaConvCfg<BN, R, S>;
  static_assert(C::SMEM <= 227 * 1024 && C::SMEM == tma_conv_smem(BN, R, S), "shared memory");
  auto kern = k_conv3x3_tma<BN, R, S>;
  static std::atomic<unsigned long long> attr_done{0};
  if (fd::ensure_smem_attr(kern, 227 * 1024, attr_done) != cudaSuccess)
    return fd::check_launch("sg_conv3x3_tma: shared-memory attribute");
  // no more CTAs per SM than their tensor memory columns fit (512): a larger
  // shared-memory request keeps the others off the SM instead of blocking in
  // tcgen05.alloc
  int smem = C::SMEM;
  const int fit = 512 / C::COLS;
  if (kSmPerSmBytes / (smem + 1024) > fit) smem = kSmPerSmBytes / (fit + 1) - 1024 + 1;
  if (smem > 227 * 1024) smem = 227 * 1024;
  ConvMaps maps;
  if (int r = encode_conv_maps(maps, x, N, H, W, Cin, w, Cout, R, BN)) return r;
  dim3 grid((unsigned)((long long)N * (H / R) * (W / kTcBM)), (unsigned)(Cout / BN));
  kern<<<grid, kTcThreads, smem, s>>>(maps, H, W, Cin, b, Cout, act, z, y);
  return fd::check_launch("sg_conv3x3_tma");
}

// Tiles of at most 64 output channels are paired (with SG_TMA_PAIR): two CTAs
// share an SM, one's epilogue running while the other multiplies (measured
// on the surrogate's layers: 64 -> 64 channels 346 vs 283 TFLOP/s, 96 -> 32
// 293 vs 222); 128-channel tiles keep one CTA with four rows (two CTAs of
// 128 x 4 accumulators would not fit the tensor memory, and two rows lose:
// 384 -> 128 channels 524 vs 612 TFLOP/s).
template <int BN>
constexpr bool tma_paired() {
  return SG_TMA_PAIR && BN <= 64;
}

// Stages: one for a single chunk; two or three where paired CTAs fit an SM,
// else as many as fit one CTA (up to four).
template <int BN, int R>
int launch_tma_s(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
                 bf16* z, bf16* y, cudaStream_t s) {
  const int nk = Cin / 16;
  if (nk == 1) return launch_tma_r<BN, R, 1>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  constexpr int pair = kSmPerSmBytes / 2 - 1024;
  if constexpr (tma_paired<BN>() && tma_conv_smem(BN, R, 2) <= pair) {
    if constexpr (tma_conv_smem(BN, R, 3) <= pair) {
      if (nk >= 3) return launch_tma_r<BN, R, 3>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
    }
    return launch_tma_r<BN, R, 2>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  } else {
    if constexpr (tma_conv_smem(BN, R, 4) <= 227 * 1024) {
      if (nk >= 4) return launch_tma_r<BN, R, 4>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
    }
    if constexpr (tma_conv_smem(BN, R, 3) <= 227 * 1024) {
      if (nk >= 3) return launch_tma_r<BN, R, 3>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
    }
    return launch_tma_r<BN, R, 2>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  }
}

// rows per CTA: four where the height allows, else two or one
template <int BN>
int launch_tma(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
               bf16* z, bf16* y, cudaStream_t s) {
  if (H % 4 == 0) return launch_tma_s<BN, 4>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  if (H % 2 == 0) return launch_tma_s<BN, 2>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  return launch_tma_s<BN, 1>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
}

// ---------------------------------------------------------------------------
// Persistent, warp-specialised variant (sg_conv3x3_tma_ws).  The CTA keeps
// two accumulator buffers of R x BN TMEM columns and walks its tiles (tile =
// CTA index + k x grid; the output-channel tiles of a pixel tile are
// consecutive, so CTAs that run at the same time share the input halo through
// L2).  Warp 8 (one thread) issues the boxes and MMAs of the CTA's chunk
// sequence (tile j, chunk kc) -> c = j x nk + kc through the same ring of S
// stages, the ring running on across tile boundaries; after a tile's last
// MMAs it commits the tile's accumulator buffer to accf[j % 2].  Warps 0..7
// (warp w: TMEM lanes 32 (w % 4) .. + 31 = pixels of each row, the 16-column
// groups w / 4, w / 4 + 2, ...) wait for accf, read the accumulators, add the
// bias, apply GELU, store, and arrive on acce[j % 2] (one arrival per warp);
// the MMAs of tile j + 2 wait for it.  So one tile's epilogue overlaps the
// next tile's MMAs and the next tiles' loads.
// ---------------------------------------------------------------------------
#ifndef SG_WS_BN_MAX  // output channels of the persistent kernel's widest tile (128 or 64)
#define SG_WS_BN_MAX 128
#endif
constexpr int kWsEpiWarps = 8;
constexpr int kWsThreads = 32 * (kWsEpiWarps + 1);

template <int BN, int R, int S>
struct WsCfg : TmaStage<BN, R> {
  static constexpr int OFF_BAR = S * TmaStage<BN, R>::STAGE;
  static constexpr int SMEM = OFF_BAR + (2 * S + 4) * 8 + 16 + 128;
  static constexpr int NCOL = 2 * R * BN;  // two accumulator buffers
  static constexpr int COLS = NCOL <= 32 ? 32 : (NCOL <= 64 ? 64 : (NCOL <= 128 ? 128 : (NCOL <= 256 ? 256 : 512)));
  static_assert(NCOL <= 512, "two accumulator buffers in tensor memory");
};

constexpr int ws_conv_smem(int BN, int R, int S) {
  return S * (2 * (((R + 2) * kHaloPx * 16 + 127) / 128 * 128) + 18 * BN * 16) + (2 * S + 4) * 8 + 16 + 128;
}

template <int BN, int R, int S>
__global__ void __launch_bounds__(kWsThreads, 1) k_conv3x3_tma_ws(const __grid_constant__ ConvMaps maps, int N, int H,
                                                                 int W, int Cin, const float* __restrict__ bias,
                                                                 int Cout, int act, bf16* __restrict__ z,
                                                                 bf16* __restrict__ y) {
  using C = TmaStage<BN, R>;
  using WC = WsCfg<BN, R, S>;
  extern __shared__ char smem_raw[];
  char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + WC::OFF_BAR);
  uint64_t* empty = full + S;
  uint64_t* accf = empty + S;  // [2]
  uint64_t* acce = accf + 2;   // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tiles_x = W / kTcBM;
  const int nco = Cout / BN;
  const int ntiles = N * (H / R) * tiles_x * nco;
  const int nk = Cin / 16;
  const int mine = blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;  // tiles of this CTA

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(WC::COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < 2 * S + 2; ++i) mbar_init(&full[i]);  // full, empty, accf: one arrival each
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acce[0])), "n"(kWsEpiWarps) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acce[1])), "n"(kWsEpiWarps) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // tile j of this CTA -> (first output row n*H + yy, x0, co0)
  auto tile_of = [&](int j, int& row, int& x0, int& co0) {
    const int t = (int)blockIdx.x + j * (int)gridDim.x;
    const int pt = t / nco;
    co0 = (t % nco) * BN;
    x0 = (pt % tiles_x) * kTcBM;
    row = (pt / tiles_x) * R;
  };

  if (warp == kWsEpiWarps) {
    if (lane == 0) {
      const int nc = mine * nk;  // chunks of this CTA
      int pend_full[S], pend_empty[S];
#pragma unroll
      for (int i = 0; i < S; ++i) pend_full[i] = pend_empty[i] = -1;
      auto issue = [&](int c, int st) {
        int row, x0, co0;
        tile_of(c / nk, row, x0, co0);
        const int kc = c % nk, n = row / H, yy = row % H;
        char* As = smem + st * C::STAGE;
        char* Bs = As + C::A_BYTES;
        mbar_expect_tx(&full[st], (unsigned)C::TX);
#pragma unroll
        for (int s = 0; s < 2; ++s) tma_load_4d(As + s * C::SLICE, &maps.x, kc * 16 + 8 * s, x0 - 1, yy - 1, n, &full[st]);
#pragma unroll
        for (int tap = 0; tap < 9; ++tap)
#pragma unroll
          for (int s = 0; s < 2; ++s)
            tma_load_3d(Bs + tap * C::TB + s * C::BSL, &maps.w, kc * 16 + 8 * s, tap, co0, &full[st]);
        pend_full[st] = c;
      };
      constexpr uint32_t idesc = instr_desc<kTcBM, BN>();
      bool ok = true;
      for (int c = 0; c < S && c < nc; ++c) issue(c, c);
      for (int c = 0; c < nc && ok; ++c) {
        const int j = c / nk, kc = c % nk, b = j & 1, st = c % S;
        if (kc == 0 && j >= 2) {  // buffer b: the epilogue of tile j - 2 has read it
          ok = mbar_wait_ok(&acce[b], (unsigned)((j - 2) >> 1) & 1u, true);
          if (!ok) break;
        }
        ok = mbar_wait_ok(&full[st], (unsigned)(c / S) & 1u, true);
        if (!ok) break;
        pend_full[st] = -1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a0 = smem_u32(smem + st * C::STAGE), b0 = a0 + C::A_BYTES;
        const uint32_t d0 = tmem + (uint32_t)(b * R * BN);
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
          const int ky = tap / 3, kx = tap % 3;
          const uint64_t bd = smem_desc(b0 + tap * C::TB, C::BSL, 128);
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const uint64_t ad = smem_desc(a0 + (r + ky) * C::ROWB + kx * 16, C::SLICE, 128);
            tc_mma(d0 + (uint32_t)(r * BN), ad, bd, idesc, (kc > 0 || tap > 0) ? 1u : 0u);
          }
        }
        tc_commit(&empty[st]);
        pend_empty[st] = c;
        if (kc == nk - 1) tc_commit(&accf[b]);  // tile j's accumulators are complete
        if (c >= 1 && c - 1 + S < nc) {        // refill the stage of chunk c-1
          const int ps = (c - 1) % S;
          ok = mbar_wait_ok(&empty[ps], (unsigned)((c - 1) / S) & 1u, true);
          if (!ok) break;
          pend_empty[ps] = -1;
          issue(c - 1 + S, ps);
        }
      }
#pragma unroll
      for (int i = 0; i < S; ++i) {
        if (pend_full[i] >= 0) mbar_wait_ok(&full[i], (unsigned)(pend_full[i] / S) & 1u, false);
        if (pend_empty[i] >= 0) mbar_wait_ok(&empty[i], (unsigned)(pend_empty[i] / S) & 1u, false);
      }
    }
    __syncwarp();
  } else {
    // epilogue: warp w reads TMEM lanes 32 q .. 32 q + 31 (pixels x0 + 32 q + lane of each row, q = w % 4),
    // 16-column groups h, h + 2, ... (h = w / 4)
    const int q = warp & 3, h = warp >> 2;
    for (int j = 0; j < mine; ++j) {
      const int b = j & 1;
      int row, x0, co0;
      tile_of(j, row, x0, co0);
      mbar_wait_ok(&accf[b], (unsigned)(j >> 1) & 1u, true);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
      for (int r = 0; r < R; ++r) {
        const long long p = ((long long)(row + r) * W + x0) + q * 32 + lane;
#pragma unroll
        for (int c0 = 16 * h; c0 < BN; c0 += 32) {
          float v[16];
          tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * R * BN + r * BN + c0), v);
          const int co = co0 + c0;
          uint32_t zw[8], yw[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            float t0 = v[2 * i] + (bias ? bias[co + 2 * i] : 0.0f);
            float t1 = v[2 * i + 1] + (bias ? bias[co + 2 * i + 1] : 0.0f);
            const __nv_bfloat162 zp = __floats2bfloat162_rn(t0, t1);
            zw[i] = *reinterpret_cast<const uint32_t*>(&zp);
            if (act == SG_ACT_GELU) {
              t0 = gelu_f(t0);
              t1 = gelu_f(t1);
            }
            const __nv_bfloat162 yp = __floats2bfloat162_rn(t0, t1);
            yw[i] = *reinterpret_cast<const uint32_t*>(&yp);
          }
          const size_t o = (size_t)p * Cout + co;
          if (z) {
            reinterpret_cast<uint4*>(z + o)[0] = make_uint4(zw[0], zw[1], zw[2], zw[3]);
            reinterpret_cast<uint4*>(z + o)[1] = make_uint4(zw[4], zw[5], zw[6], zw[7]);
          }
          if (y) {
            reinterpret_cast<uint4*>(y + o)[0] = make_uint4(yw[0], yw[1], yw[2], yw[3]);
            reinterpret_cast<uint4*>(y + o)[1] = make_uint4(yw[4], yw[5], yw[6], yw[7]);
          }
        }
      }
      // this warp's reads of buffer b are complete (tcgen05.wait::ld in tmem_ld16)
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acce[b])) : "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(WC::COLS) : "memory");
  }
}

template <int BN, int R, int S>
int launch_ws_r(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
                bf16* z, bf16* y, cudaStream_t s) {
  using WC = WsCfg<BN, R, S>;
  static_assert(WC::SMEM <= 227 * 1024 && WC::SMEM == ws_conv_smem(BN, R, S), "shared memory");
  auto kern = k_conv3x3_tma_ws<BN, R, S>;
  static std::atomic<unsigned long long> attr_done{0};
  if (fd::ensure_smem_attr(kern, 227 * 1024, attr_done) != cudaSuccess)
    return fd::check_launch("sg_conv3x3_tma_ws: shared-memory attribute");
  int smem = WC::SMEM;
  const int fit = 512 / WC::COLS;  // CTAs per SM whose accumulators fit the tensor memory
  if (kSmPerSmBytes / (smem + 1024) > fit) smem = kSmPerSmBytes / (fit + 1) - 1024 + 1;
  if (smem > 227 * 1024) smem = 227 * 1024;
  int per_sm = 1, dev = 0, sms = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWsThreads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long ntiles = (long long)N * (H / R) * (W / kTcBM) * (Cout / BN);
  const long long grid = std::min<long long>(ntiles, (long long)sms * per_sm);
  ConvMaps maps;
  if (int r = encode_conv_maps(maps, x, N, H, W, Cin, w, Cout, R, BN)) return r;
  kern<<<(unsigned)grid, kWsThreads, smem, s>>>(maps, N, H, W, Cin, b, Cout, act, z, y);
  return fd::check_launch("sg_conv3x3_tma_ws");
}

// the most stages (up to six) that fit one CTA
template <int BN, int R>
int launch_ws_s(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
                bf16* z, bf16* y, cudaStream_t s) {
  if constexpr (ws_conv_smem(BN, R, 6) <= 227 * 1024) return launch_ws_r<BN, R, 6>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  else if constexpr (ws_conv_smem(BN, R, 5) <= 227 * 1024) return launch_ws_r<BN, R, 5>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  else return launch_ws_r<BN, R, 4>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
}

// rows per tile: the most of 4, 2, 1 that divide H with two buffers of R x BN
// accumulator columns in the tensor memory
template <int BN>
int launch_ws(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
              bf16* z, bf16* y, cudaStream_t s) {
  if constexpr (2 * 4 * BN <= 512) {
    if (H % 4 == 0) return launch_ws_s<BN, 4>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  }
  if (H % 2 == 0) return launch_ws_s<BN, 2>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  return launch_ws_s<BN, 1>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
}

// ---------------------------------------------------------------------------
// Weight gradient on tcgen05 (sg_conv3x3_wgrad_tc):
//   dw[co][tap][ci] = sum_p dz[p][co] x[p + (ky-1, kx-1)][ci]
// as D[co][ci] (M = 128 output channels, N = BN input channels, K = pixels)
// per tap.  A CTA takes one kernel row ky (its three taps kx = 0..2, three
// accumulators of BN TMEM columns), one output-channel tile, one input-channel
// tile and a contiguous range of pixel chunks (128 pixels of one image row).
// Both operands are channel-contiguous in memory, so they are MN-major (in
// the matrix descriptor of an MN-major operand without swizzle, as of a
// K-major one, LBO is the stride between core matrices along K and SBO the
// stride between 8-row groups along M or N; the other reading of the two
// fields fails the GPU tests):
//   A: a dz box (8 channels x 128 pixels) per 8-channel group below Cout ->
//      [pixel][8 channels], core matrices of 8 pixels 128 B apart along K
//      (LBO), groups 2048 B apart (SBO); the groups at or beyond Cout are
//      zeroed once and never loaded;
//   B: an x box (8 channels x 130 pixels of row y + ky - 1) per 8-channel
//      group, groups kWgBGrp apart (SBO); tap kx is the window 16 B x kx
//      into it.
// One thread issues the boxes of a ring of S stages and the 3 x 8 MMAs of a
// chunk; the FP32 partial sums go to partial[split][co][tap][ci] and are
// added in a fixed order afterwards, so the result does not depend on
// scheduling.
// ---------------------------------------------------------------------------
constexpr int kWgBGrp = ((kHaloPx * 16 + 127) / 128) * 128;  // 2176 B: one 8-channel group of the x halo

template <int BN, bool SW>
struct WgTcCfg {
  // SW: the input channels on M (x halo as A, dz as B), else the output channels
  static constexpr int AGRP = SW ? kWgBGrp : 2048;          // bytes of one 8-channel group of A
  static constexpr int BGRP = SW ? 2048 : kWgBGrp;          // and of B
  static constexpr int A_BYTES = 16 * AGRP;                 // 128 channels
  static constexpr int B_BYTES = (BN / 8) * BGRP;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int S = (227 * 1024 - 1024) / STAGE > 5 ? 5 : (227 * 1024 - 1024) / STAGE;
  static constexpr int OFF_BAR = S * STAGE;
  static constexpr int SMEM = OFF_BAR + 2 * S * 8 + 16 + 128;
  static constexpr int NCOL = 3 * BN;
  static constexpr int COLS = NCOL <= 32 ? 32 : (NCOL <= 64 ? 64 : (NCOL <= 128 ? 128 : (NCOL <= 256 ? 256 : 512)));
  static_assert(BN % 16 == 0 && BN >= 16 && BN <= 128 && S >= 2, "tile");
  static_assert(STAGE % 128 == 0 && AGRP % 128 == 0 && BGRP % 128 == 0, "128-byte aligned boxes");
};

// instruction descriptor of kind::f16 with both operands MN-major (transpose bits 15 and 16)
template <int M, int N>
__device__ __forceinline__ constexpr uint32_t instr_desc_mn() {
  return instr_desc<M, N>() | (1u << 15) | (1u << 16);
}

template <int BN, bool SW>
__global__ void __launch_bounds__(kTcThreads, 1) k_wgrad_tc(const __grid_constant__ ConvMaps maps, int N, int H,
                                                           int W, int Cin, int Cout, int cps, long long nchunks,
                                                           float* __restrict__ partial) {
  using C = WgTcCfg<BN, SW>;
  constexpr int S = C::S;
  extern __shared__ char smem_raw[];
  char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
  uint64_t* empty = full + S;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(empty + S);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128, n0 = blockIdx.y * BN;  // first channel on M and on N
  const int co0 = SW ? n0 : m0, ci0 = SW ? m0 : n0;
  const int mch = SW ? Cin : Cout;                        // channels on M
  const int ky = blockIdx.z % 3, split = blockIdx.z / 3;
  const long long c0 = (long long)split * cps;
  const int nc = (int)(c0 < nchunks ? (nchunks - c0 < cps ? nchunks - c0 : cps) : 0);
  const int tiles_x = W / kTcBM;
  const int ngrp = (mch - m0) / 8 < 16 ? (mch - m0) / 8 : 16;  // A channel groups loaded

  // the A channel groups at or beyond the channel count stay zero in every stage
  constexpr int GV = C::AGRP / 16;
  for (int i = tid; i < S * (16 - ngrp) * GV; i += kTcThreads) {
    const int st = i / ((16 - ngrp) * GV), rem = i % ((16 - ngrp) * GV);
    reinterpret_cast<uint4*>(smem + st * C::STAGE + ngrp * C::AGRP)[rem] = make_uint4(0u, 0u, 0u, 0u);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(C::COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < 2 * S; ++i) mbar_init(&full[i]);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (tid == 0 && nc > 0) {
    int pend_full[S], pend_empty[S];
#pragma unroll
    for (int i = 0; i < S; ++i) pend_full[i] = pend_empty[i] = -1;
    // dz boxes: 8 output channels x 128 pixels; x boxes: 8 input channels x 130 pixels of row y + ky - 1
    const int ndz = SW ? BN / 8 : ngrp, nx = SW ? ngrp : BN / 8;
    const unsigned tx = (unsigned)(ndz * 2048 + nx * kHaloPx * 16);
    auto issue = [&](int c, int st) {
      const long long g = c0 + c;
      const int x0 = (int)(g % tiles_x) * kTcBM;
      const long long rowg = g / tiles_x;
      const int n = (int)(rowg / H), y = (int)(rowg % H);
      char* As = smem + st * C::STAGE;
      char* Bs = As + C::A_BYTES;
      char* dzs = SW ? Bs : As;
      char* xs = SW ? As : Bs;
      constexpr int DZG = SW ? C::BGRP : C::AGRP, XG = SW ? C::AGRP : C::BGRP;
      mbar_expect_tx(&full[st], tx);
      for (int j = 0; j < ndz; ++j) tma_load_4d(dzs + j * DZG, &maps.w, co0 + 8 * j, x0, y, n, &full[st]);
      for (int j = 0; j < nx; ++j) tma_load_4d(xs + j * XG, &maps.x, ci0 + 8 * j, x0 - 1, y + ky - 1, n, &full[st]);
      pend_full[st] = c;
    };
    constexpr uint32_t idesc = instr_desc_mn<kTcBM, BN>();
    bool ok = true;
    for (int c = 0; c < S && c < nc; ++c) issue(c, c);
    for (int c = 0; c < nc && ok; ++c) {
      const int st = c % S;
      ok = mbar_wait_ok(&full[st], (unsigned)(c / S) & 1u, true);
      if (!ok) break;
      pend_full[st] = -1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t a0 = smem_u32(smem + st * C::STAGE), b0 = a0 + C::A_BYTES;
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        // tap kx: the x halo window starts kx pixels (16 B each) into its boxes
        const uint32_t ash = SW ? (uint32_t)(kx * 16) : 0u, bsh = SW ? 0u : (uint32_t)(kx * 16);
#pragma unroll
        for (int s8 = 0; s8 < 8; ++s8) {
          const uint64_t ad = smem_desc(a0 + ash + s8 * 256, 128, C::AGRP);
          const uint64_t bd = smem_desc(b0 + bsh + s8 * 256, 128, C::BGRP);
          tc_mma(tmem + (uint32_t)(kx * BN), ad, bd, idesc, (c > 0 || s8 > 0) ? 1u : 0u);
        }
      }
      tc_commit(&empty[st]);
      pend_empty[st] = c;
      if (c >= 1 && c - 1 + S < nc) {
        const int ps = (c - 1) % S;
        ok = mbar_wait_ok(&empty[ps], (unsigned)((c - 1) / S) & 1u, true);
        if (!ok) break;
        pend_empty[ps] = -1;
        issue(c - 1 + S, ps);
      }
    }
#pragma unroll
    for (int i = 0; i < S; ++i) {
      if (pend_full[i] >= 0) mbar_wait_ok(&full[i], (unsigned)(pend_full[i] / S) & 1u, false);
      if (pend_empty[i] >= 0) mbar_wait_ok(&empty[i], (unsigned)(pend_empty[i] / S) & 1u, false);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  // epilogue: warp w holds channels m0 + 32 w + lane of M (TMEM lanes), BN channels of N per tap
  const int m = m0 + warp * 32 + lane;
  float* out = partial + (size_t)split * Cout * 9 * Cin;
#pragma unroll 1
  for (int kx = 0; kx < 3; ++kx) {
    const int tap = ky * 3 + kx;
#pragma unroll
    for (int cc = 0; cc < BN; cc += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(kx * BN + cc), v);
      if (nc == 0) {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = 0.0f;
      }
      if (m < mch) {
        if constexpr (SW) {  // m = input channel, columns = output channels n0 + cc ..
#pragma unroll
          for (int i = 0; i < 16; ++i) out[((size_t)(n0 + cc + i) * 9 + tap) * Cin + m] = v[i];
        } else {             // m = output channel, columns = input channels n0 + cc ..
          float* o = out + ((size_t)m * 9 + tap) * Cin + n0 + cc;
#pragma unroll
          for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(o + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::COLS) : "memory");
  }
}

__global__ void k_wg_sum(const float* __restrict__ partial, int splits, size_t n, float* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int k = 0; k < splits; ++k) s += partial[(size_t)k * n + i];
  out[i] = s;
}

// Tensor maps of the weight gradient: x (C, W, H, N) with boxes of 8
// channels x 130 pixels x 1 row, dz (Cout, W, H, N) with boxes of 8 channels x
// 128 pixels x 1 row (kept in ConvMaps::w).
inline int encode_wgrad_maps(ConvMaps& m, const bf16* x, const bf16* dz, int N, int H, int W, int Cin, int Cout) {
  const fd::EncodeTiledFn fn = fd::encode_tiled_fn();
  FD_REQUIRE(fn != nullptr, FD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint32_t e4[4] = {1u, 1u, 1u, 1u};
  const cuuint64_t xd[4] = {(cuuint64_t)Cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
  const cuuint64_t xs[3] = {(cuuint64_t)Cin * 2, (cuuint64_t)W * Cin * 2, (cuuint64_t)H * W * Cin * 2};
  const cuuint32_t xb[4] = {8u, (cuuint32_t)kHaloPx, 1u, 1u};
  CUresult r = fn(&m.x, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(x), xd, xs, xb, e4,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  FD_REQUIRE(r == CUDA_SUCCESS, FD_ERR_CUDA, "sg_conv3x3_wgrad_tc: input tensor map (%d)", (int)r);
  const cuuint64_t dd[4] = {(cuuint64_t)Cout, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
  const cuuint64_t ds[3] = {(cuuint64_t)Cout * 2, (cuuint64_t)W * Cout * 2, (cuuint64_t)H * W * Cout * 2};
  const cuuint32_t db[4] = {8u, (cuuint32_t)kTcBM, 1u, 1u};
  r = fn(&m.w, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(dz), dd, ds, db, e4,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  FD_REQUIRE(r == CUDA_SUCCESS, FD_ERR_CUDA, "sg_conv3x3_wgrad_tc: gradient tensor map (%d)", (int)r);
  return FD_OK;
}

template <int BN, bool SW>
int launch_wgrad_tc(const bf16* x, const bf16* dz, int N, int H, int W, int Cin, int Cout, float* dw, float* partial,
                    size_t partial_floats, int splits, cudaStream_t s) {
  using C = WgTcCfg<BN, SW>;
  static_assert(C::SMEM <= 227 * 1024, "shared memory");
  auto kern = k_wgrad_tc<BN, SW>;
  static std::atomic<unsigned long long> attr_done{0};
  if (fd::ensure_smem_attr(kern, 227 * 1024, attr_done) != cudaSuccess)
    return fd::check_launch("sg_conv3x3_wgrad_tc: shared-memory attribute");
  const long long nchunks = (long long)N * H * (W / kTcBM);
  const int m_t = ((SW ? Cin : Cout) + 127) / 128, n_t = (SW ? Cout : Cin) / BN;
  const size_t n = (size_t)Cout * 9 * Cin;
  if (splits <= 0) {  // the most CTAs that fill two waves of one CTA per SM, within the chunks and the buffer
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long per = (long long)m_t * n_t * 3;
    splits = (int)std::max<long long>(1, (2LL * sms) / per);
  }
  if ((long long)splits > nchunks) splits = (int)nchunks;
  if ((size_t)splits * n > partial_floats) splits = (int)(partial_floats / n);
  FD_REQUIRE(splits >= 1, FD_ERR_ARG, "sg_conv3x3_wgrad_tc: partial buffer too small");
  const int cps = (int)((nchunks + splits - 1) / splits);
  ConvMaps maps;
  if (int r = encode_wgrad_maps(maps, x, dz, N, H, W, Cin, Cout)) return r;
  dim3 grid((unsigned)m_t, (unsigned)n_t, (unsigned)(3 * splits));
  kern<<<grid, kTcThreads, C::SMEM, s>>>(maps, N, H, W, Cin, Cout, cps, nchunks, partial);
  k_wg_sum<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(partial, splits, n, dw);
  return fd::check_launch("sg_conv3x3_wgrad_tc");
}

template <int BN, int BK, int R>
int launch_tch_r(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
                 bf16* z, bf16* y, cudaStream_t s) {
  using C = HaloCfg<BN, BK, R>;
  auto kern = k_conv3x3_tch<BN, BK, R>;
  static std::atomic<unsigned long long> attr_done{0};
  if (fd::ensure_smem_attr(kern, C::SMEM, attr_done) != cudaSuccess)
    return fd::check_launch("sg_conv3x3_tc: shared-memory attribute");
  dim3 grid((unsigned)((long long)N * (H / R) * (W / kTcBM)), (unsigned)(Cout / BN));
  kern<<<grid, kTcThreads, C::SMEM, s>>>(x, N, H, W, Cin, w, b, Cout, act, z, y);
  return fd::check_launch("sg_conv3x3_tc");
}

// rows per CTA: four where the height allows (the weights of a chunk then
// serve 512 pixels), else two or one
template <int BN, int BK>
int launch_tch(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
               bf16* z, bf16* y, cudaStream_t s) {
  if (H % 4 == 0) return launch_tch_r<BN, BK, 4>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  if (H % 2 == 0) return launch_tch_r<BN, BK, 2>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  return launch_tch_r<BN, BK, 1>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
}

template <int BN, int BK>
int launch_tc(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act,
              bf16* z, bf16* y, cudaStream_t s) {
  using C = TcCfg<BN, BK>;
  auto kern = k_conv3x3_tc<BN, BK>;
  static std::atomic<unsigned long long> attr_done{0};
  if (fd::ensure_smem_attr(kern, C::SMEM, attr_done) != cudaSuccess)
    return fd::check_launch("sg_conv3x3_tc: shared-memory attribute");
  const long long M = (long long)N * H * W;
  dim3 grid((unsigned)((M + kTcBM - 1) / kTcBM), (unsigned)(Cout / BN));
  kern<<<grid, kTcThreads, C::SMEM, s>>>(x, N, H, W, Cin, w, b, Cout, act, z, y);
  return fd::check_launch("sg_conv3x3_tc");
}

template <int BK>
int tc_bk(const bf16* x, int N, int H, int W, int Cin, const bf16* w, const float* b, int Cout, int act, bf16* z,
          bf16* y, cudaStream_t s) {
  if (Cout % 64 == 0) return launch_tc<64, BK>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  if (Cout % 32 == 0) return launch_tc<32, BK>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
  return launch_tc<16, BK>(x, N, H, W, Cin, w, b, Cout, act, z, y, s);
}

}  // namespace
}  // namespace sg

extern "C" {

int sg_conv3x3_tc(const void* x, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout, int act,
                  void* z, void* y, void* stream) {
  FD_REQUIRE(x && w && (z || y) && N > 0 && H > 0 && W > 0, FD_ERR_ARG, "sg_conv3x3_tc: bad arguments");
  FD_REQUIRE(Cin % 16 == 0 && Cout % 16 == 0 && Cin > 0 && Cout > 0, FD_ERR_SHAPE,
             "sg_conv3x3_tc: channel counts must be positive multiples of 16 (got %d -> %d)", Cin, Cout);
  FD_REQUIRE(act == SG_ACT_NONE || act == SG_ACT_GELU, FD_ERR_ARG, "sg_conv3x3_tc: activation %d", act);
  FD_REQUIRE(((uintptr_t)x | (uintptr_t)w | (uintptr_t)z | (uintptr_t)y) % 16 == 0, FD_ERR_ARG,
             "sg_conv3x3_tc: tensors must be 16-byte aligned");
  using sg::bf16;
  cudaStream_t s = fd::as_stream(stream);
  const bf16 *xb = (const bf16*)x, *wb = (const bf16*)w;
  if (W % sg::kTcBM == 0) {  // halo tiles: the input is read once per tile
    bf16 *zb = (bf16*)z, *yb = (bf16*)y;
    if (Cin % 32 == 0) {
      if (Cout % 64 == 0) return sg::launch_tch<64, 32>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
      if (Cout % 32 == 0) return sg::launch_tch<32, 32>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
      return sg::launch_tch<16, 32>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
    }
    if (Cout % 64 == 0) return sg::launch_tch<64, 16>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
    if (Cout % 32 == 0) return sg::launch_tch<32, 16>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
    return sg::launch_tch<16, 16>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
  }
  if (Cin % 64 == 0) return sg::tc_bk<64>(xb, N, H, W, Cin, wb, bias, Cout, act, (bf16*)z, (bf16*)y, s);
  if (Cin % 32 == 0) return sg::tc_bk<32>(xb, N, H, W, Cin, wb, bias, Cout, act, (bf16*)z, (bf16*)y, s);
  return sg::tc_bk<16>(xb, N, H, W, Cin, wb, bias, Cout, act, (bf16*)z, (bf16*)y, s);
}

int sg_conv3x3_tma(const void* x, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout,
                   int act, void* z, void* y, void* stream) {
  FD_REQUIRE(x && w && (z || y) && N > 0 && H > 0 && W > 0, FD_ERR_ARG, "sg_conv3x3_tma: bad arguments");
  FD_REQUIRE(W % sg::kTcBM == 0 && Cin % 16 == 0 && Cout % 16 == 0 && Cin > 0 && Cout > 0, FD_ERR_SHAPE,
             "sg_conv3x3_tma: needs W a multiple of 128 and channel counts multiples of 16 (got W=%d, %d -> %d)", W,
             Cin, Cout);
  FD_REQUIRE(act == SG_ACT_NONE || act == SG_ACT_GELU, FD_ERR_ARG, "sg_conv3x3_tma: activation %d", act);
  FD_REQUIRE(((uintptr_t)x | (uintptr_t)w | (uintptr_t)z | (uintptr_t)y) % 16 == 0, FD_ERR_ARG,
             "sg_conv3x3_tma: tensors must be 16-byte aligned");
  using sg::bf16;
  cudaStream_t s = fd::as_stream(stream);
  const bf16 *xb = (const bf16*)x, *wb = (const bf16*)w;
  bf16 *zb = (bf16*)z, *yb = (bf16*)y;
  if (SG_TMA_BN_MAX >= 128 && Cout % 128 == 0) return sg::launch_tma<128>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
  if (Cout % 64 == 0) return sg::launch_tma<64>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
  if (Cout % 32 == 0) return sg::launch_tma<32>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
  return sg::launch_tma<16>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
}

int sg_conv3x3_tma_ws(const void* x, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout,
                      int act, void* z, void* y, void* stream) {
  FD_REQUIRE(x && w && (z || y) && N > 0 && H > 0 && W > 0, FD_ERR_ARG, "sg_conv3x3_tma_ws: bad arguments");
  FD_REQUIRE(W % sg::kTcBM == 0 && Cin % 16 == 0 && Cout % 16 == 0 && Cin > 0 && Cout > 0, FD_ERR_SHAPE,
             "sg_conv3x3_tma_ws: needs W a multiple of 128 and channel counts multiples of 16 (got W=%d, %d -> %d)",
             W, Cin, Cout);
  FD_REQUIRE(act == SG_ACT_NONE || act == SG_ACT_GELU, FD_ERR_ARG, "sg_conv3x3_tma_ws: activation %d", act);
  FD_REQUIRE(((uintptr_t)x | (uintptr_t)w | (uintptr_t)z | (uintptr_t)y) % 16 == 0, FD_ERR_ARG,
             "sg_conv3x3_tma_ws: tensors must be 16-byte aligned");
  using sg::bf16;
  cudaStream_t s = fd::as_stream(stream);
  const bf16 *xb = (const bf16*)x, *wb = (const bf16*)w;
  bf16 *zb = (bf16*)z, *yb = (bf16*)y;
  if (SG_WS_BN_MAX >= 128 && Cout % 128 == 0) return sg::launch_ws<128>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
  if (Cout % 64 == 0) return sg::launch_ws<64>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
  if (Cout % 32 == 0) return sg::launch_ws<32>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
  return sg::launch_ws<16>(xb, N, H, W, Cin, wb, bias, Cout, act, zb, yb, s);
}

int sg_conv3x3_wgrad_tc(const void* x, const void* dz, int N, int H, int W, int Cin, int Cout, float* dw,
                        float* partial, size_t partial_floats, int splits, void* stream) {
  FD_REQUIRE(x && dz && dw && partial && N > 0 && H > 0 && W > 0, FD_ERR_ARG, "sg_conv3x3_wgrad_tc: bad arguments");
  FD_REQUIRE(W % sg::kTcBM == 0 && Cin % 16 == 0 && Cout % 16 == 0 && Cin > 0 && Cout > 0, FD_ERR_SHAPE,
             "sg_conv3x3_wgrad_tc: needs W a multiple of 128 and channel counts multiples of 16 (got W=%d, %d -> %d)",
             W, Cin, Cout);
  FD_REQUIRE(((uintptr_t)x | (uintptr_t)dz | (uintptr_t)dw | (uintptr_t)partial) % 16 == 0, FD_ERR_ARG,
             "sg_conv3x3_wgrad_tc: tensors must be 16-byte aligned");
  using sg::bf16;
  cudaStream_t s = fd::as_stream(stream);
  const bf16 *xb = (const bf16*)x, *db = (const bf16*)dz;
  // the larger channel count on M (128 rows of the MMA), the other on N
  if (Cin > Cout) {
    if (Cout % 128 == 0) return sg::launch_wgrad_tc<128, true>(xb, db, N, H, W, Cin, Cout, dw, partial, partial_floats, splits, s);
    if (Cout % 64 == 0) return sg::launch_wgrad_tc<64, true>(xb, db, N, H, W, Cin, Cout, dw, partial, partial_floats, splits, s);
    if (Cout % 32 == 0) return sg::launch_wgrad_tc<32, true>(xb, db, N, H, W, Cin, Cout, dw, partial, partial_floats, splits, s);
    return sg::launch_wgrad_tc<16, true>(xb, db, N, H, W, Cin, Cout, dw, partial, partial_floats, splits, s);
  }
  if (Cin % 128 == 0) return sg::launch_wgrad_tc<128, false>(xb, db, N, H, W, Cin, Cout, dw, partial, partial_floats, splits, s);
  if (Cin % 64 == 0) return sg::launch_wgrad_tc<64, false>(xb, db, N, H, W, Cin, Cout, dw, partial, partial_floats, splits, s);
  if (Cin % 32 == 0) return sg::launch_wgrad_tc<32, false>(xb, db, N, H, W, Cin, Cout, dw, partial, partial_floats, splits, s);
  return sg::launch_wgrad_tc<16, false>(xb, db, N, H, W, Cin, Cout, dw, partial, partial_floats, splits, s);
}

int sg_tc_status(unsigned* out, int clear) {
  FD_REQUIRE(out != nullptr, FD_ERR_ARG, "sg_tc_status: NULL pointer");
  if (cudaMemcpyFromSymbol(out, sg::g_sg_tc_error, sizeof(unsigned)) != cudaSuccess)
    return fd::check_launch("sg_tc_status");
  if (clear) {
    const unsigned zero = 0;
    if (cudaMemcpyToSymbol(sg::g_sg_tc_error, &zero, sizeof(unsigned)) != cudaSuccess)
      return fd::check_launch("sg_tc_status");
  }
  return FD_OK;
}

}  // extern "C"
