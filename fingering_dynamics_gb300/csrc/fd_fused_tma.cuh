// Fused step, packed deviation storage, with rows staged in shared memory by
// bulk asynchronous copies (cp.async.bulk, completion on mbarriers).
//
// A CTA of NT threads owns a band of NT consecutive cells of every row of a
// strip of R rows and marches down the strip.  Shared memory holds a ring of
// row slots; a slot holds one lattice row of all 18 population planes for the
// band plus a 16-byte halo on each side.  One thread issues the bulk copies of
// rows ahead while the CTA works on row y, so global-memory latency is covered
// by the rows in flight instead of by warps waiting on loads.  Two rings:
//   NS >= 5 whole-row slots (with the mask row), one mbarrier each; row
//     y + NS - 2 is issued at row y (FP16 / BF16 storage);
//   NS == 4 split slots whose f half and g half complete on separate
//     mbarriers and are refilled as soon as each is no longer read, with the
//     mask rows in a ring of their own (FP32 storage: the smaller footprint
//     fits 5 CTAs per SM instead of 4).
//
// Per row y, each thread (one cell x = x0 + t):
//   1. pulls g of row y+1 from the ring (stream + bounce-back + Zou-He g,
//      fingering_periodic.py:327-343, bounce_back.py, fingering_periodic.py:278-302),
//      forms psi(y+1) (fingering_periodic.py:210-212) and writes it to a
//      4-row psi ring (threads 0 and 1 also do the halo cells x0-1, x0+NT);
//   2. __syncthreads: psi(y+1) complete, row y-2 no longer read;
//   3. reads the 3x3 psi neighbourhood, pulls f of row y, applies Zou-He f,
//      forms the macroscopic fields and collides (fingering_periodic.py:455-479),
//      and stores the new populations to global memory.
// Rows are loaded with wrap-around in y (the reference's np.roll); the band's
// halo beyond the lattice's x edges is not loaded because the populations
// streamed across x = 0 and x = W-1 are replaced by the Zou-He rules before use.
#pragma once

#include "fd_fused_dev.cuh"
#include "fd_host.h"
#include "fd_tmap.h"

// Band width (threads per CTA) of the single-lattice launch, and ring depth
// per storage type for both launches (NS == 4: the split ring; NS >= 5:
// whole-row slots).  Measured on 4096 x 2048: FP32 (memory-bound) gains 9% on
// the split ring, which fits 5 CTAs per SM instead of 4; FP16/BF16
// (issue-bound) lose 5% on it and keep five whole-row slots.
#ifndef FD_TMA_NT
#define FD_TMA_NT 128
#endif
#ifndef FD_TMA_NS_F32
#define FD_TMA_NS_F32 4
#endif
#ifndef FD_TMA_NS_16
#define FD_TMA_NS_16 5
#endif
// 1: the single-lattice kernel walks the odd strips of the split ring from
// their top row down, so neighbouring strips (launched close together) read
// their shared halo rows at about the same time; 0: every strip walks up.
// Same results either way.  The batch kernel always walks up: its tiles come
// from a counter, largest first, and walking down measured 1.9% slower on the
// 96-member ensemble (36,188 vs 36,874 MLUPS) while the single lattice gains
// 0.6% (DRAM reads 694 -> 630 MB per launch on 4096 x 2048).
#ifndef FD_TMA_WALK_DOWN
#define FD_TMA_WALK_DOWN 1
#endif

namespace fd {

template <typename SF>
constexpr int tma_ring_depth() {
  return std::is_same_v<SF, float> ? FD_TMA_NS_F32 : FD_TMA_NS_16;
}

// FP32 storage carries psi as a float pair hi + lo (fd_dev.cuh, dev_psi_pair)
// through the psi ring; the lo parts (at most half an ulp of hi) are kept as
// FP16 scaled by 2^24, whose 11-bit significand leaves an error below 1e-11.
template <typename SF>
constexpr bool psi_paired() {
  return std::is_same_v<SF, float>;
}
constexpr float kPsiLoScale = 16777216.0f;          // 2^24
constexpr float kPsiLoInv = 1.0f / 16777216.0f;

constexpr unsigned kWaitLimit = 1u << 24;  // bounded spins on an mbarrier

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// One box of a 3-D tensor map (coordinates x, row, plane) into shared memory
// (128-byte aligned destination; x * element size a multiple of 16 bytes).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Wait for phase `parity` of an mbarrier, at most `limit` polls.  Returns
// false (and latches the device error word) if the phase never completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned limit = kWaitLimit) {
  const uint32_t a = smem_u32(bar);
  for (unsigned it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  atomicOr(&g_fd_device_error, kStatusWaitTimeout);
  return false;
}

// Byte layout of one ring slot for a band of NT cells: the nine f plane rows,
// the eight g_i plane rows (from a 128-byte boundary: both blocks are
// tensor-map boxes), the FP32 g_0 row and the mask row.  TENSOR: a band row
// of an SF plane fits one box (at most 256 cells); wider bands copy each
// plane row with a 1-D bulk copy.
template <typename SF, int NT>
struct SlotLayout {
  static constexpr int HF = 16 / (int)sizeof(SF);     // halo elements of an SF plane
  static constexpr int HG = 4;                        // halo elements of the FP32 g_0 plane
  static constexpr int HM = 8;                        // halo elements of the uint16 mask row
  static constexpr int RF = ((NT + 2 * HF) * (int)sizeof(SF) + 15) / 16 * 16;
  static constexpr int RG = ((NT + 2 * HG) * 4 + 15) / 16 * 16;
  static constexpr int RM = ((NT + 2 * HM) * 2 + 15) / 16 * 16;
  static constexpr bool TENSOR = NT + 2 * HF <= 256;
  static_assert(RF == (NT + 2 * HF) * (int)sizeof(SF), "a plane row is one dense box row");
  static constexpr int OFF_GI = (9 * RF + 127) / 128 * 128;
  static constexpr int OFF_G0 = OFF_GI + 8 * RF;
  static constexpr int OFF_M = OFF_G0 + RG;
  static constexpr int BYTES = (OFF_M + RM + 127) / 128 * 128;
  // tensor-map boxes land on 128-byte boundaries, bulk copies on 16-byte ones
  static_assert(OFF_GI % 128 == 0 && OFF_G0 % 128 == 0 && OFF_M % 16 == 0 && RM % 16 == 0, "slot alignment");
  static_assert(!TENSOR || NT + 2 * HG <= 256, "the g_0 row fits one box when the SF rows do");
};

// Shared memory of the staged kernel.  NS >= 5: a ring of NS whole-row slots
// (f, g and mask of a row behind one mbarrier).  NS == 4: the split ring, four
// slots whose f half and g half complete on separate mbarriers (0..3: g half
// and mask row, 4..7: f half), without the mask; the mask rows live in a ring
// of their own and arrive with the g half (6 rows: row r arrives at the
// barrier of row r - 4 and is last read by the f pull of row r).  The psi ring
// holds 4 rows of NT + 2 floats, plus their FP16 lo parts when psi is paired;
// with the 6-row mask ring the FP32 split ring still fits five CTAs per SM.
template <typename SF, int NT, int NS>
struct TmaSmem {
  using L = SlotLayout<SF, NT>;
  static constexpr bool SPLIT = NS == 4;
  static constexpr int NBAR = SPLIT ? 8 : NS;
  static constexpr int PSI_ROW = NT + 2;
  static constexpr int OFF_BAR = 0;
  static constexpr int OFF_PSI = 128;
  static constexpr int OFF_PLO = OFF_PSI + 4 * PSI_ROW * 4;
  static constexpr int OFF_MASK = (OFF_PLO + (psi_paired<SF>() ? 4 * PSI_ROW * 2 : 0) + 127) / 128 * 128;
  static constexpr int MASK_ROWS = SPLIT ? 6 : 0;
  static constexpr int OFF_SLOT = (OFF_MASK + MASK_ROWS * L::RM + 127) / 128 * 128;
  static constexpr int SLOT = SPLIT ? (L::OFF_M + 127) / 128 * 128 : L::BYTES;
  static constexpr int BYTES = OFF_SLOT + NS * SLOT;
  static constexpr int ALLOC = BYTES + 128;  // dynamic shared memory: BYTES from a 128-byte boundary
  static_assert(NBAR * 8 <= OFF_PSI, "mbarriers overlap the psi ring");
  static_assert(OFF_SLOT % 128 == 0 && SLOT % 128 == 0 && OFF_MASK % 16 == 0, "slots on 128-byte boundaries");
};

// The 128-byte aligned start of the dynamic shared memory.
__device__ __forceinline__ char* smem_aligned(char* raw) {
  return raw + ((128u - (smem_u32(raw) & 127u)) & 127u);
}

// The part of lattice row r (wrapped into [0, H)) that a band loads: per kind
// of plane the first loaded cell, the bytes per plane row and the byte offset
// of the first loaded cell within the slot row (the band's halo is clipped at
// the lattice's x edges).
template <typename SF, int NT>
struct RowSpan {
  size_t rowoff;
  int y;  // the row, wrapped into [0, H)
  int xs, gs, ms;
  unsigned nf, ng, nm;
  int df, dg, dm;
  __device__ __forceinline__ RowSpan(int r, int x0, int H, int W) {
    using L = SlotLayout<SF, NT>;
    y = wrap(r, H);
    rowoff = (size_t)y * W;
    xs = max(x0 - L::HF, 0);
    gs = max(x0 - L::HG, 0);
    ms = max(x0 - L::HM, 0);
    nf = (unsigned)((min(x0 + NT + L::HF, W) - xs) * (int)sizeof(SF));
    ng = (unsigned)((min(x0 + NT + L::HG, W) - gs) * 4);
    nm = (unsigned)((min(x0 + NT + L::HM, W) - ms) * 2);
    df = (xs - (x0 - L::HF)) * (int)sizeof(SF);
    dg = (gs - (x0 - L::HG)) * 4;
    dm = (ms - (x0 - L::HM)) * 2;
  }
};

// Bytes one SF plane row of the band brings into its slot: a whole box row
// (cells beyond the lattice's x edges read as zero) or the clipped span.
template <typename SF, int NT>
__device__ __forceinline__ unsigned plane_row_bytes(const RowSpan<SF, NT>& s) {
  if constexpr (SlotLayout<SF, NT>::TENSOR) return (unsigned)SlotLayout<SF, NT>::RF;
  else return s.nf;
}

// The nine f plane rows: one tensor-map box, or a bulk copy per plane.
template <typename SF, int NT>
__device__ __forceinline__ void copy_f_half(const DevArgs<SF>& a, const TmaMaps* tm, char* slot, uint64_t* bar,
                                            const RowSpan<SF, NT>& s, int x0) {
  using L = SlotLayout<SF, NT>;
  if constexpr (L::TENSOR) {
    tma_load_3d(slot, &tm->f, x0 - L::HF, s.y, 0, bar);
  } else {
#pragma unroll
    for (int i = 0; i < 9; ++i)
      bulk_g2s(slot + i * L::RF + s.df, a.src_f + i * a.pstride_f + s.rowoff + s.xs, s.nf, bar);
  }
}

// Bytes the FP32 g_0 row of the band brings into its slot.
template <typename SF, int NT>
__device__ __forceinline__ unsigned g0_row_bytes(const RowSpan<SF, NT>& s) {
  if constexpr (SlotLayout<SF, NT>::TENSOR) return (unsigned)SlotLayout<SF, NT>::RG;
  else return s.ng;
}

// The eight g_i plane rows and the FP32 g_0 row: one box each, or a bulk copy
// per plane.
template <typename SF, int NT>
__device__ __forceinline__ void copy_g_half(const DevArgs<SF>& a, const TmaMaps* tm, char* slot, uint64_t* bar,
                                            const RowSpan<SF, NT>& s, int x0) {
  using L = SlotLayout<SF, NT>;
  if constexpr (L::TENSOR) {
    tma_load_3d(slot + L::OFF_G0, &tm->g0, x0 - L::HG, s.y, 0, bar);
    tma_load_3d(slot + L::OFF_GI, &tm->gi, x0 - L::HF, s.y, 0, bar);
  } else {
    bulk_g2s(slot + L::OFF_G0 + s.dg, a.src_g0 + s.rowoff + s.gs, s.ng, bar);
#pragma unroll
    for (int i = 0; i < 8; ++i)
      bulk_g2s(slot + L::OFF_GI + i * L::RF + s.df, a.src_gi + i * a.pstride_f + s.rowoff + s.xs, s.nf, bar);
  }
}

// Issue the copies of lattice row r into a whole-row slot (NS >= 5).
template <typename SF, int NT>
__device__ __forceinline__ void issue_row(const DevArgs<SF>& a, const TmaMaps* tm, char* slot, uint64_t* bar, int r,
                                          int x0) {
  using L = SlotLayout<SF, NT>;
  const RowSpan<SF, NT> s(r, x0, a.H, a.W);
  mbar_expect_tx(bar, 17 * plane_row_bytes(s) + g0_row_bytes(s) + s.nm);
  copy_f_half<SF, NT>(a, tm, slot, bar, s, x0);
  copy_g_half<SF, NT>(a, tm, slot, bar, s, x0);
  bulk_g2s(slot + L::OFF_M + s.dm, a.mask + s.rowoff + s.ms, s.nm, bar);
}

// Split ring (NS == 4): the g half of row r with its mask row, and the f half.
template <typename SF, int NT>
__device__ __forceinline__ void issue_g_half(const DevArgs<SF>& a, const TmaMaps* tm, char* slot, char* mrow,
                                             uint64_t* bar, int r, int x0) {
  const RowSpan<SF, NT> s(r, x0, a.H, a.W);
  mbar_expect_tx(bar, 8 * plane_row_bytes(s) + g0_row_bytes(s) + s.nm);
  copy_g_half<SF, NT>(a, tm, slot, bar, s, x0);
  bulk_g2s(mrow + s.dm, a.mask + s.rowoff + s.ms, s.nm, bar);
}

template <typename SF, int NT>
__device__ __forceinline__ void issue_f_half(const DevArgs<SF>& a, const TmaMaps* tm, char* slot, uint64_t* bar,
                                             int r, int x0) {
  const RowSpan<SF, NT> s(r, x0, a.H, a.W);
  mbar_expect_tx(bar, 9 * plane_row_bytes(s));
  copy_f_half<SF, NT>(a, tm, slot, bar, s, x0);
}

// Shared-memory load of element idx of a plane row at byte offset `off` from
// the shared-memory base, converted to FP32 (times `scale` for scaled storage).
template <typename S, bool SCALED>
__device__ __forceinline__ float sld(const char* sm, int off, int idx, float scale) {
  const S v = reinterpret_cast<const S*>(sm + off)[idx];
  if constexpr (std::is_same_v<S, float>) return v;
  else if constexpr (SCALED) return to_f<S>(v) * scale;
  else return to_f<S>(v);
}

// Pulled populations of band cell lx (may be -1 or NT) of row y.  rows[k]
// is the byte offset of the slot of row y - 1 + k.  Plane i comes from row
// y - ey_i at lx - ex_i; bounce-back links replace it by the opposite plane
// of the same cell (bounce_back.py).
template <typename SF, int NT, bool IS_G, bool SCALED>
__device__ __forceinline__ void pull_cell(const char* sm, const DevCoef& c, const int (&rows)[3], int lx,
                                          unsigned bits, float (&v)[9]) {
  using L = SlotLayout<SF, NT>;
  const float s = IS_G ? c.inv_sg : c.inv_sf;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const int row = rows[1 - ey_of(i)];
    if (IS_G && i == 0) v[0] = sld<float, false>(sm, row + L::OFF_G0, lx + L::HG, 1.0f);
    else if (IS_G) v[i] = sld<SF, SCALED>(sm, row + L::OFF_GI + (i - 1) * L::RF, lx - ex_of(i) + L::HF, s);
    else v[i] = sld<SF, SCALED>(sm, row + i * L::RF, lx - ex_of(i) + L::HF, s);
  }
  if (bits) {
#pragma unroll
    for (int i = 1; i < 9; ++i) {
      if (bits & (1u << (i - 1))) {
        const int o = opp_of(i);
        if (IS_G) v[i] = sld<SF, SCALED>(sm, rows[1] + L::OFF_GI + (o - 1) * L::RF, lx + L::HF, s);
        else v[i] = sld<SF, SCALED>(sm, rows[1] + o * L::RF, lx + L::HF, s);
      }
    }
  }
}

// Mask word of band cell lx; `mrow` is the byte offset of the mask row.
template <typename SF, int NT>
__device__ __forceinline__ unsigned mask_at(const char* sm, int mrow, int lx) {
  using L = SlotLayout<SF, NT>;
  return reinterpret_cast<const uint16_t*>(sm + mrow)[lx + L::HM];
}

// psi of cell x (band index lx) of row y from its pulled g after Zou-He
// (fingering_periodic.py:210-212, 278-302); the pulled g is returned in g.
// `mrow` is the byte offset of row y's mask row.

// Stores of one cell's new populations into the packed layout (q = y W + x).
// FP16/BF16: the 17 values in the storage type (f_0..f_8 then g_1..g_8) are
// converted two at a time with one instruction (pair_from_f, pair_from_f_sr:
// one 32-bit random word per pair) and written as 16-bit stores; g_0 stays FP32.
template <typename SF, bool SCALED, bool STOCH>
__device__ __forceinline__ void store_cell(const DevArgs<SF>& a, size_t q, const float (&f)[9], const float (&g)[9]) {
  if constexpr (std::is_same_v<SF, float>) {
    float* pf = a.dst_f + q;
#pragma unroll
    for (int i = 0; i < 9; ++i, pf += a.pstride_f) *pf = f[i];
    a.dst_g0[q] = g[0];
    float* pg = a.dst_gi + q;
#pragma unroll
    for (int i = 1; i < 9; ++i, pg += a.pstride_f) *pg = g[i];
  } else {
    float v[18];
#pragma unroll
    for (int i = 0; i < 9; ++i) v[i] = SCALED ? f[i] * a.c.sf : f[i];
#pragma unroll
    for (int i = 1; i < 9; ++i) v[8 + i] = SCALED ? g[i] * a.c.sg : g[i];
    v[17] = 0.0f;
    uint32_t rs = 0;
    if constexpr (STOCH) rs = sr_hash((uint32_t)q ^ a.seed);
    auto plane = [&](int k) -> uint16_t* {
      SF* p = k < 9 ? a.dst_f + (size_t)k * a.pstride_f + q : a.dst_gi + (size_t)(k - 9) * a.pstride_f + q;
      return reinterpret_cast<uint16_t*>(p);
    };
#pragma unroll
    for (int k = 0; k < 17; k += 2) {
      uint32_t w;
      if constexpr (STOCH) {
        rs = sr_next(rs);
        w = pair_from_f_sr<SF>(v[k], v[k + 1], rs);
      } else {
        w = pair_from_f<SF>(v[k], v[k + 1]);
      }
      *plane(k) = (uint16_t)w;
      if (k + 1 < 17) *plane(k + 1) = (uint16_t)(w >> 16);
    }
    a.dst_g0[q] = g[0];
  }
}

// With paired psi (psi_paired) the result is the pair (hi, lo), else (psi, 0).
template <typename SF, int NT, bool SCALED>
__device__ __forceinline__ float2 psi_cell(const char* sm, const DevArgs<SF>& a, const int (&rows)[3], int mrow, int x,
                                           int lx, int y, float (&g)[9]) {
  if (x < 0) return make_float2(1.0f, 0.0f);
  if (x >= a.W) return make_float2(-1.0f, 0.0f);
  const unsigned m = mask_at<SF, NT>(sm, mrow, lx);
  pull_cell<SF, NT, true, SCALED>(sm, a.c, rows, lx, m & 0xFFu, g);
  if (x == 0 || x == a.W - 1) dev_zou_he_g(a.c, a.variant, a.H, a.W, x, y, g);
  if (m & SOLID) return make_float2(a.c.psi_wall, 0.0f);
  if constexpr (psi_paired<SF>()) {
    return dev_psi_pair(g);
  } else {  // 16-bit storage: the sum on direction pairs in packed FP32x2 arithmetic (dev_collide_x2)
    const float2 s = __fadd2_rn(__fadd2_rn(make_float2(g[1], g[2]), make_float2(g[3], g[4])),
                                __fadd2_rn(make_float2(g[5], g[6]), make_float2(g[7], g[8])));
    return make_float2(g[0] + (s.x + s.y), 0.0f);
  }
}

// The psi ring (4 rows of NT + 2 cells, hi parts as floats, lo parts as scaled
// FP16 when psi is paired).  `row` is the element offset of a ring row.
template <typename SF, int NT, int NS>
struct PsiRing {
  float* hi;
  __half* lo;
  __device__ __forceinline__ explicit PsiRing(char* smem)
      : hi(reinterpret_cast<float*>(smem + TmaSmem<SF, NT, NS>::OFF_PSI)),
        lo(reinterpret_cast<__half*>(smem + TmaSmem<SF, NT, NS>::OFF_PLO)) {}
  __device__ __forceinline__ void put(int row, int j, float2 v) const {
    hi[row + j] = v.x;
    if constexpr (psi_paired<SF>()) lo[row + j] = __float2half_rn(v.y * kPsiLoScale);
  }
  __device__ __forceinline__ float2 get(int row, int j) const {
    if constexpr (psi_paired<SF>()) return make_float2(hi[row + j], __half2float(lo[row + j]) * kPsiLoInv);
    else return make_float2(hi[row + j], 0.0f);
  }
};

// Stencils of cell j of the psi ring row `pc` (rows pm and pn below and
// above); the cell's own column comes from registers (S, C, N).
template <typename SF, int NT, int NS>
__device__ __forceinline__ DevStencil ring_stencil(const PsiRing<SF, NT, NS>& ring, int pm, int pc, int pn, int j,
                                                   float2 S, float2 C, float2 N) {
  if constexpr (psi_paired<SF>()) {
    return dev_stencil_pair(C, ring.get(pc, j + 1), ring.get(pc, j - 1), N, S, ring.get(pn, j + 1),
                            ring.get(pn, j - 1), ring.get(pm, j + 1), ring.get(pm, j - 1));
  } else {
    const float* h = ring.hi;
    return dev_stencil(C.x, h[pc + j + 1], h[pc + j - 1], N.x, S.x, h[pn + j + 1], h[pn + j - 1], h[pm + j + 1],
                       h[pm + j - 1]);
  }
}

// One strip of one band: the body shared by the single-lattice kernel and the
// batched persistent kernel.  The mbarriers must be initialised; `phase`
// (per-slot parity of the next fill to wait for) and `ok` carry over from
// strip to strip.  Ends with a CTA barrier, so the ring can be refilled.
template <typename SF, int NT, int NS, bool SCALED, bool STOCH>
__device__ __forceinline__ void tma_strip_ring(const DevArgs<SF>& a, const TmaMaps* tm, int band, int strip, char* smem,
                                               unsigned& phase, bool& ok) {
  static_assert(NS >= 5, "rows y-2 .. y+2 must be resident while row y is computed");
  using L = SlotLayout<SF, NT>;
  using M = TmaSmem<SF, NT, NS>;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + M::OFF_BAR);
  const PsiRing<SF, NT, NS> ring(smem);
  const float2 wallv = make_float2(a.c.psi_wall, 0.0f);

  const int t = threadIdx.x;
  const int x0 = band * NT;
  const int y0 = strip * a.R, y1 = min(y0 + a.R, a.H);
  const int x = x0 + t;
  const bool owned = x < a.W;
  const bool walls = a.variant == FD_VARIANT_WALLS;
  const int first = y0 - 2, last = y1 + 1;  // ring rows: y0-2 .. y1+1
  // halo cells of the band: the left one by thread NT/2, the right one by
  // the last thread (warp 0 issues the copies; other warps take the halos)
  const int hl = (t == NT / 2) ? -1 : (t == NT - 1 ? NT : 0);
  const bool halo = (t == NT / 2) || (t == NT - 1);

  // row first + k lives in slot k (mod NS); rows y0-2 .. y0+NS-3 fill slots 0..NS-1
  if (t == 0) {
    for (int k = 0; k < NS && first + k <= last; ++k)
      issue_row<SF, NT>(a, tm, smem + M::OFF_SLOT + k * M::SLOT, &bars[k], first + k, x0);
  }
  auto wait_slot = [&](int s) {
    if (ok) ok = mbar_wait(&bars[s], (phase >> s) & 1u);
    phase ^= 1u << s;
  };
  // slots of rows y-2 .. y+NS-3 (rotated every row) and their byte offsets
  int si[NS], so[NS];
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    si[k] = k;  // rows y0-2 .. y0+NS-3
    so[k] = M::OFF_SLOT + k * M::SLOT;
  }
  int pslot = 0;  // psi ring slot of row y0-1; rows y0-1, y0, y0+1 use pslot, +1, +2 (mod 4)
  auto psi_row = [&](int k) { return ((pslot + k) & 3) * M::PSI_ROW; };

  float gC[9], gN[9];
  float2 pS = wallv, pC = wallv;  // psi of this column at rows y-1 and y
  bool bad = false;               // a fluid cell with a non-finite rho or psi
  // prologue: psi of rows y0-1 and y0 (needs rows y0-2 .. y0+1)
  wait_slot(0);
  wait_slot(1);
  wait_slot(2);
  wait_slot(3);
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int r = y0 - 1 + k;
    const int rows[3] = {so[k], so[k + 1], so[k + 2]};
    const int pr = psi_row(k);
    const bool ghost = walls && (r < 0 || r >= a.H);
    const int yr = wrap(r, a.H);
    const float2 pv = ghost ? wallv : psi_cell<SF, NT, SCALED>(smem, a, rows, rows[1] + L::OFF_M, x, t, yr, gN);
    ring.put(pr, t + 1, pv);
    if (k == 0) pS = pv;
    else pC = pv;
    if (halo) {
      float gh[9];
      ring.put(pr, hl + 1,
               ghost ? wallv : psi_cell<SF, NT, SCALED>(smem, a, rows, rows[1] + L::OFF_M, x0 + hl, hl, yr, gh));
    }
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) gC[i] = gN[i];

  for (int y = y0; y < y1; ++y) {
    // 1. psi of row y+1 from rows y, y+1, y+2
    float2 pN;
    wait_slot(si[4]);
    {
      const int rows[3] = {so[2], so[3], so[4]};
      const bool ghost = walls && (y + 1 >= a.H);
      const int yr = wrap(y + 1, a.H);
      const int pr = psi_row(2);
      pN = ghost ? wallv : psi_cell<SF, NT, SCALED>(smem, a, rows, rows[1] + L::OFF_M, x, t, yr, gN);
      ring.put(pr, t + 1, pN);
      if (halo) {
        float gh[9];
        ring.put(pr, hl + 1,
                 ghost ? wallv : psi_cell<SF, NT, SCALED>(smem, a, rows, rows[1] + L::OFF_M, x0 + hl, hl, yr, gh));
      }
    }
    // rho_inlet - 1 of row 1 (bottom inlet corner, rows 0..2 = y..y+2) or of
    // row H-2 (top inlet corner, rows H-3..H-1 = y-2..y) for the walled
    // variant (fingering.py:341, 357); row y-2 is recycled after the barrier.
    float drho_nb = 0.0f;
    if (walls && x == 0 && (y == 0 || y == a.H - 1)) {
      const int prow[3] = {y == 0 ? so[2] : so[0], y == 0 ? so[3] : so[1], y == 0 ? so[4] : so[2]};
      const int yn = (y == 0) ? 1 : a.H - 2;
      float fn[9];
      pull_cell<SF, NT, false, SCALED>(smem, a.c, prow, t, mask_at<SF, NT>(smem, prow[1] + L::OFF_M, t) & 0xFFu, fn);
      drho_nb = dev_inlet_drho(fn, (float)a.inlet_ux[yn], a.side_in[0 * a.H + yn], a.side_in[2 * a.H + yn]);
    }
    // 2. psi(y+1) complete; the slot of row y-2 is free for row y+NS-2
    __syncthreads();
    if (t == 0 && y + NS - 2 <= last) issue_row<SF, NT>(a, tm, smem + so[0], &bars[si[0]], y + NS - 2, x0);
    // 3. stencils, f pull, Zou-He, collision, store
    if (owned) {
      const DevStencil st = ring_stencil(ring, psi_row(0), psi_row(1), psi_row(2), t + 1, pS, pC, pN);
      const int rows[3] = {so[1], so[2], so[3]};
      const unsigned m = mask_at<SF, NT>(smem, rows[1] + L::OFF_M, t);
      float f[9];
      pull_cell<SF, NT, false, SCALED>(smem, a.c, rows, t, m & 0xFFu, f);
      if (x == 0 || x == a.W - 1) {
        const int o = (x == 0) ? 0 : 3;
        dev_zou_he_f(a.c, a.variant, a.H, a.W, x, y, f, (float)a.inlet_ux[y], a.side_in[(o + 0) * a.H + y],
                     a.side_in[(o + 1) * a.H + y], a.side_in[(o + 2) * a.H + y], drho_nb);
        a.side_out[(o + 0) * a.H + y] = st.gx;
        a.side_out[(o + 1) * a.H + y] = st.gy;
        a.side_out[(o + 2) * a.H + y] = dev_mu(a.c, st);
      }
      if (!(m & SOLID)) {
        const DevMacro mc = dev_macros<!std::is_same_v<SF, float>>(a.c, f, st);
        bad |= nonfinite_cell(mc.rho, mc.psi);
        dev_collide_for<SF>(a.c, mc, f, gC);
      }
      store_cell<SF, SCALED, STOCH>(a, (size_t)y * a.W + x, f, gC);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) gC[i] = gN[i];
    pS = pC;
    pC = pN;
    // rotate: rows y-1 .. y+NS-2 become y-2 .. y+NS-3 for the next row
    const int freed = si[0], freed_off = so[0];
#pragma unroll
    for (int k = 0; k < NS - 1; ++k) {
      si[k] = si[k + 1];
      so[k] = so[k + 1];
    }
    si[NS - 1] = freed;
    so[NS - 1] = freed_off;
    pslot = (pslot + 1) & 3;
  }
  // After a wait gave up, make sure the last copy issued into every slot has
  // landed (bounded) before the ring is reused or released.
  if (!ok && t == 0) {
    for (int s = 0; s < NS; ++s) {
      const int span = last - first;
      if (span < s) continue;
      const int k = span - ((span - s) % NS);  // last ring row (relative) filled into slot s
      mbar_wait(&bars[s], (unsigned)((k / NS) & 1));
    }
  }
  if (__syncthreads_or(bad) && t == 0) report_nonfinite(a);
  ok = __syncthreads_and(ok);
}

// rho_inlet - 1 of row yn (1 or H-2) of the walled variant's inlet column
// (fingering.py:341, 357) from f pulled straight from global memory.  Only the
// directions dev_inlet_drho reads (e_x <= 0) are loaded; the others stay 0.
template <typename SF, bool SCALED>
__device__ __forceinline__ float inlet_corner_drho(const DevArgs<SF>& a, int yn) {
  const unsigned bits = a.mask[(size_t)yn * a.W] & 0xFFu;
  auto ld = [&](int i, int y, int x) -> float {
    const SF v = a.src_f[(size_t)i * a.pstride_f + (size_t)y * a.W + x];
    if constexpr (std::is_same_v<SF, float>) return v;
    else if constexpr (SCALED) return to_f<SF>(v) * a.c.inv_sf;
    else return to_f<SF>(v);
  };
  float d[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    if (i > 0 && (bits & (1u << (i - 1)))) d[i] = ld(opp_of(i), yn, 0);
    else if (ex_of(i) > 0) d[i] = 0.0f;
    else d[i] = ld(i, wrap(yn - ey_of(i), a.H), -ex_of(i));
  }
  return dev_inlet_drho(d, (float)a.inlet_ux[yn], a.side_in[yn], a.side_in[2 * a.H + yn]);
}

// The strip on the split ring (NS == 4).  Row r of the strip's ring rows
// y0-2 .. y1+1 uses slot (r - first) & 3; its g half (g_0 and the eight g_i
// planes, needed by psi of rows r-1 .. r+1) and its f half (needed by the f
// pull of rows r-1 .. r+1) complete on separate mbarriers, so each half is
// refilled as soon as it is no longer read: the g half of row y+4 and the f
// half of row y+2 are issued at the barrier of row y, 1.5 and 1 rows ahead of
// their first use.  The mask row of r (needed up to the f pull of row r)
// arrives with the g half into mask-ring row (r - first) % 6.  The f half of
// row y0-2 is never needed (the inlet corners read global memory), so the
// prologue fills f rows y0-1 .. y0+2.
//
// `down` walks the strip from its top row to its bottom row instead: the
// ring schedule is the same in the strip's own row order (local row l is
// lattice row y0 + l going up, y1 - 1 - l going down), and the cell update
// takes its rows and psi values in lattice order, so the results are the same
// bit for bit.  Odd strips walk down (FD_TMA_WALK_DOWN): the two strips that
// share a boundary then read its halo rows at about the same time (both at
// their start, or both at their end) and the second read finds them in L2.
template <typename SF, int NT, bool SCALED, bool STOCH>
__device__ __forceinline__ void tma_strip_split(const DevArgs<SF>& a, const TmaMaps* tm, int band, int strip,
                                                bool down, char* smem, unsigned& phase, bool& ok) {
  using L = SlotLayout<SF, NT>;
  using M = TmaSmem<SF, NT, 4>;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + M::OFF_BAR);
  const PsiRing<SF, NT, 4> ring(smem);
  const float2 wallv = make_float2(a.c.psi_wall, 0.0f);

  const int t = threadIdx.x;
  const int x0 = band * NT;
  const int y0 = strip * a.R, y1 = min(y0 + a.R, a.H);
  const int n = y1 - y0;  // local rows -2 .. n+1: g halves -2 .. n+1, f halves -1 .. n
  const int x = x0 + t;
  const bool owned = x < a.W;
  const bool walls = a.variant == FD_VARIANT_WALLS;
  const int hl = (t == NT / 2) ? -1 : (t == NT - 1 ? NT : 0);
  const bool halo = (t == NT / 2) || (t == NT - 1);

  auto lat = [&](int l) { return down ? y1 - 1 - l : y0 + l; };  // lattice row of local row l
  auto slot = [&](int l) { return M::OFF_SLOT + ((l + 2) & 3) * M::SLOT; };
  auto mrow = [&](int l) { return M::OFF_MASK + (int)((unsigned)(l + 2) % (unsigned)M::MASK_ROWS) * L::RM; };
  // slots of the lattice rows below, at and above local row l
  auto rows_of = [&](int l, int (&rows)[3]) {
    rows[0] = slot(down ? l + 1 : l - 1);
    rows[1] = slot(l);
    rows[2] = slot(down ? l - 1 : l + 1);
  };
  // parity bits of the fills issued (thread 0), for the error path
  unsigned issued = phase;
  auto issue_g = [&](int l) {
    if (l > n + 1 || !ok) return;
    const int b = (l + 2) & 3;
    issue_g_half<SF, NT>(a, tm, smem + slot(l), smem + mrow(l), &bars[b], lat(l), x0);
    issued ^= 1u << b;
  };
  auto issue_f = [&](int l) {
    if (l > n || !ok) return;
    const int b = 4 + ((l + 2) & 3);
    issue_f_half<SF, NT>(a, tm, smem + slot(l), &bars[b], lat(l), x0);
    issued ^= 1u << b;
  };
  auto wait_bar = [&](int b) {
    if (ok) ok = mbar_wait(&bars[b], (phase >> b) & 1u);
    phase ^= 1u << b;
  };
  auto wait_g = [&](int l) { wait_bar((l + 2) & 3); };
  auto wait_f = [&](int l) { wait_bar(4 + ((l + 2) & 3)); };

  if (t == 0) {
    for (int l = -2; l < 2; ++l) issue_g(l);
    for (int l = -1; l < 3; ++l) issue_f(l);
  }
  int pslot = 0;  // psi ring slot of local row -1; local rows -1, 0, 1 use pslot, +1, +2 (mod 4)
  auto psi_row = [&](int k) { return ((pslot + k) & 3) * M::PSI_ROW; };
  // psi of local row l (this thread's cell and its halo cell) into psi ring row k
  float gN[9];
  auto psi_of_row = [&](int l, int k) {
    int rows[3];
    rows_of(l, rows);
    const int r = lat(l);
    const bool ghost = walls && (r < 0 || r >= a.H);
    const int yr = wrap(r, a.H);
    const int pr = psi_row(k);
    const float2 pv = ghost ? wallv : psi_cell<SF, NT, SCALED>(smem, a, rows, mrow(l), x, t, yr, gN);
    ring.put(pr, t + 1, pv);
    if (halo) {
      float gh[9];
      ring.put(pr, hl + 1, ghost ? wallv : psi_cell<SF, NT, SCALED>(smem, a, rows, mrow(l), x0 + hl, hl, yr, gh));
    }
    return pv;
  };

  // prologue: psi of local rows -1 and 0; the g halves of local rows -2 and
  // -1 are refilled (local rows 2, 3) as soon as each is done
  wait_g(-2);
  wait_g(-1);
  wait_g(0);
  float2 pP = psi_of_row(-1, 0);  // psi of this column at local rows l-1 and l
  bool bad = false;               // a fluid cell with a non-finite rho or psi
  __syncthreads();
  if (t == 0) issue_g(2);
  wait_g(1);
  float2 pC = psi_of_row(0, 1);
  float gC[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) gC[i] = gN[i];
  __syncthreads();
  if (t == 0) issue_g(3);
  wait_f(-1);
  wait_f(0);

  for (int l = 0; l < n; ++l) {
    const int y = lat(l);
    // 1. psi of local row l+1 from the g halves of local rows l, l+1, l+2
    wait_g(l + 2);
    const float2 pX = psi_of_row(l + 1, 2);
    float drho_nb = 0.0f;
    if (walls && x == 0 && (y == 0 || y == a.H - 1)) drho_nb = inlet_corner_drho<SF, SCALED>(a, y == 0 ? 1 : a.H - 2);
    // 2. psi(l+1) complete: the g half of local row l and the f half of local
    //    row l-2 are free (the f half of local row 2 was filled by the prologue)
    __syncthreads();
    if (t == 0) {
      issue_g(l + 4);
      if (l > 0) issue_f(l + 2);
    }
    wait_f(l + 1);
    // 3. stencils, f pull, Zou-He, collision, store (rows and psi in lattice order)
    if (owned) {
      const float2 pS = down ? pX : pP, pN = down ? pP : pX;
      const DevStencil st = ring_stencil(ring, psi_row(down ? 2 : 0), psi_row(1), psi_row(down ? 0 : 2), t + 1, pS,
                                         pC, pN);
      int rows[3];
      rows_of(l, rows);
      const unsigned m = mask_at<SF, NT>(smem, mrow(l), t);
      float f[9];
      pull_cell<SF, NT, false, SCALED>(smem, a.c, rows, t, m & 0xFFu, f);
      if (x == 0 || x == a.W - 1) {
        const int o = (x == 0) ? 0 : 3;
        dev_zou_he_f(a.c, a.variant, a.H, a.W, x, y, f, (float)a.inlet_ux[y], a.side_in[(o + 0) * a.H + y],
                     a.side_in[(o + 1) * a.H + y], a.side_in[(o + 2) * a.H + y], drho_nb);
        a.side_out[(o + 0) * a.H + y] = st.gx;
        a.side_out[(o + 1) * a.H + y] = st.gy;
        a.side_out[(o + 2) * a.H + y] = dev_mu(a.c, st);
      }
      if (!(m & SOLID)) {
        const DevMacro mc = dev_macros<!std::is_same_v<SF, float>>(a.c, f, st);
        bad |= nonfinite_cell(mc.rho, mc.psi);
        dev_collide_for<SF>(a.c, mc, f, gC);
      }
      store_cell<SF, SCALED, STOCH>(a, (size_t)y * a.W + x, f, gC);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) gC[i] = gN[i];
    pP = pC;
    pC = pX;
    pslot = (pslot + 1) & 3;
  }
  // After a wait gave up no further copies were issued; make sure the last
  // copy issued on every mbarrier has landed (bounded) before the ring is
  // reused or released.
  if (!ok && t == 0) {
    for (int b = 0; b < M::NBAR; ++b) mbar_wait(&bars[b], ((issued >> b) & 1u) ^ 1u);
  }
  if (__syncthreads_or(bad) && t == 0) report_nonfinite(a);
  ok = __syncthreads_and(ok);
}

// `down`: walk the strip from its top row (the split ring only; the
// whole-row ring always walks up).
template <typename SF, int NT, int NS, bool SCALED, bool STOCH>
__device__ __forceinline__ void tma_strip(const DevArgs<SF>& a, const TmaMaps* tm, int band, int strip, bool down,
                                          char* smem, unsigned& phase, bool& ok) {
  if constexpr (NS == 4) tma_strip_split<SF, NT, SCALED, STOCH>(a, tm, band, strip, down, smem, phase, ok);
  else tma_strip_ring<SF, NT, NS, SCALED, STOCH>(a, tm, band, strip, smem, phase, ok);
}

template <typename SF, int NT, int NS>
__device__ __forceinline__ void init_ring(char* smem) {
  using M = TmaSmem<SF, NT, NS>;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + M::OFF_BAR);
  if (threadIdx.x == 0) {
    for (int s = 0; s < M::NBAR; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// CTAs per SM that the batch kernel's shared memory admits (228 KB per SM, 1 KB
// reserved per CTA, 256 B of static shared memory).  The split ring (FP32)
// takes it as its occupancy hint, so the compiler may use the registers that
// do not lower the occupancy (87 instead of 64 with a spill: the 96-member
// ensemble +2%); the whole-row ring (FP16/BF16) measured 5% slower with the
// hint and keeps the compiler's own choice (0: no hint).
template <typename SF, int NT, int NS>
constexpr int tma_resident_ctas() {
  const int n = 233472 / (TmaSmem<SF, NT, NS>::ALLOC + 256 + 1024);
  return n < 1 ? 1 : (n > 16 ? 16 : n);
}
static_assert(FD_TMA_NS_F32 != 4 || tma_resident_ctas<float, 128, 4>() >= 5,
              "the FP32 split ring must fit five CTAs per SM");

// CTA b takes band b % nbands of strip strip0 + b / nbands.  `tm`: the tensor maps of the step's source planes
// (a grid constant: TMA reads it from the parameter space).
template <typename SF, int NT, int NS, bool SCALED, bool STOCH>
__global__ void __launch_bounds__(NT) k_fused_tma(const __grid_constant__ DevArgs<SF> a, int nbands, int strip0,
                                                  const __grid_constant__ TmaMaps tm) {
  extern __shared__ __align__(128) char smem_raw[];
  char* smem = smem_aligned(smem_raw);
  init_ring<SF, NT, NS>(smem);
  unsigned phase = 0;
  bool ok = true;
  const int strip = strip0 + (int)blockIdx.x / nbands;
  tma_strip<SF, NT, NS, SCALED, STOCH>(a, &tm, (int)blockIdx.x % nbands, strip, FD_TMA_WALK_DOWN && (strip & 1),
                                       smem, phase, ok);
}

// One lattice of a batch: its arguments and the tensor maps of its source
// planes for both ping-pong parities (in global memory, where TMA reads them).
template <typename SF>
struct BatchInst {
  DevArgs<SF> args[2];
  TmaMaps maps[2];
};

// Persistent kernel over a tile table of (instance, band, strip) entries,
// largest tiles first: each CTA takes the next untaken tile from a counter
// until none is left (greedy largest-first balancing of uneven tiles).  Every
// instance advances one iteration.
//
// `ctl` holds two two-slot counters, written so that the launch of parity p
// never writes a slot it reads and launches on a stream are ordered (the
// sequence is deterministic and advances under CUDA-graph replay too):
//   ctl[0..1]  batch steps done, for stochastic rounding: the launch reads
//              ctl[p] and one thread writes ctl[1-p] = ctl[p] + 1; a member's
//              step seed is its own seed (args.seed) plus the count;
//   ctl[2..3]  tile counter: the launch takes tiles from ctl[2+p] and one
//              thread zeroes ctl[2+(1-p)] for the next launch.
template <typename SF, int NT, int NS, bool SCALED, bool STOCH>
__global__ void __launch_bounds__(NT, (NS == 4 ? tma_resident_ctas<SF, NT, NS>() : 0)) k_fused_tma_batch(const BatchInst<SF>* __restrict__ inst,
                                                        const int4* __restrict__ tiles, int ntiles, int parity,
                                                        unsigned* __restrict__ ctl) {
  extern __shared__ __align__(128) char smem_raw[];
  __shared__ DevArgs<SF> sa;
  __shared__ const TmaMaps* stm;
  __shared__ int next;
  __shared__ int skip;
  char* smem = smem_aligned(smem_raw);
  init_ring<SF, NT, NS>(smem);
  unsigned done = 0;
  if constexpr (STOCH) done = ctl[parity];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if constexpr (STOCH) ctl[parity ^ 1] = done + 1;
    ctl[2 + (parity ^ 1)] = 0;
  }
  unsigned phase = 0;
  bool ok = true;
  for (;;) {
    if (threadIdx.x == 0) {
      next = (int)atomicAdd(&ctl[2 + parity], 1u);
      skip = 0;
      if (next < ntiles) {
        sa = inst[tiles[next].x].args[parity];
        stm = &inst[tiles[next].x].maps[parity];
        if constexpr (STOCH) sa.seed = sr_hash(sa.seed + done);
        // a quarantined member (non-finite cell seen) is not stepped any more
        skip = *reinterpret_cast<volatile unsigned*>(sa.status) != 0u;
      }
    }
    __syncthreads();
    const int k = next;
    if (k >= ntiles || !ok) break;
    if (skip) {
      __syncthreads();  // every thread has read next / skip before thread 0 rewrites them
      continue;
    }
    const int4 tl = tiles[k];
    tma_strip<SF, NT, NS, SCALED, STOCH>(sa, stm, tl.y, tl.z, false, smem, phase, ok);
  }
}

}  // namespace fd

namespace fd {

// Raise the kernel's dynamic shared-memory limit (once per device).
template <typename SF, int NT, int NS, bool SCALED, bool STOCH>
cudaError_t tma_prepare_kernel() {
  static std::atomic<unsigned long long> attr_done{0};
  return ensure_smem_attr(k_fused_tma<SF, NT, NS, SCALED, STOCH>, TmaSmem<SF, NT, NS>::ALLOC, attr_done);
}

// Tensor maps of the f, g_i and g_0 planes of the packed buffer `src` (bands of
// NT cells; unused, and left empty, when a band row does not fit one box).
template <typename SF, int NT>
int tma_maps(const DevArgs<SF>& a, const char* src, TmaMaps& m) {
  using L = SlotLayout<SF, NT>;
  m = TmaMaps{};
  if constexpr (!L::TENSOR) return FD_OK;
  const PackedLayout<SF> P = packed_layout<SF>(a.H, a.W);
  const int es = (int)sizeof(SF), box = NT + 2 * L::HF;
  const size_t pb = P.pstride * sizeof(SF);
  if (int r = encode_plane_rows(&m.f, src + P.off_f, es, a.W, a.H, 9, pb, box)) return r;
  if (int r = encode_plane_rows(&m.gi, src + P.off_gi, es, a.W, a.H, 8, pb, box)) return r;
  return encode_plane_rows(&m.g0, src + P.off_g0, 4, a.W, a.H, 1, P.off_gi - P.off_g0, NT + 2 * L::HG);
}

// Arguments of the staged kernel for one lattice with strips of R rows; the
// buffers are set per step by tma_set_step.  R <= 0 picks the strip count from
// the resident CTAs per SM (measured on 4096 x 2048): the split ring (FP32,
// memory-bound) loses up to 8% to a partial last wave and takes the largest
// count that fits in three full waves (R = 29 there: 36.8 vs 34.0 GLUPS at
// 3.1 waves); the whole-row ring (FP16/BF16, issue-bound) is best with short
// strips, about four waves (R = 16 there: 46.5 vs 45.7 GLUPS at two waves;
// 12..18 rows within 1%).
template <typename SF, int NT, int NS, bool SCALED, bool STOCH>
DevArgs<SF> tma_args(const fd_params& p, const DevCoef& c, const uint16_t* mask, const double* inlet_ux, int R) {
  using M = TmaSmem<SF, NT, NS>;
  const PackedLayout<SF> L = packed_layout<SF>(p.H, p.W);
  DevArgs<SF> a;
  a.c = c;
  a.H = p.H;
  a.W = p.W;
  a.variant = p.variant;
  a.P = L.P;
  a.pstride_f = L.pstride;
  a.mask = mask;
  a.inlet_ux = inlet_ux;
  a.status = nullptr;
  const int nbands = (p.W + NT - 1) / NT;
  if (R <= 0) {
    int per_sm = 1;
    tma_prepare_kernel<SF, NT, NS, SCALED, STOCH>();  // the occupancy depends on the raised limit
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fused_tma<SF, NT, NS, SCALED, STOCH>, NT, M::ALLOC);
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long slots = (long long)sms * (per_sm > 0 ? per_sm : 1);
    long long strips = M::SPLIT ? 3 * slots / nbands : (4 * slots + nbands - 1) / nbands;
    if (strips < 1) strips = 1;
    R = (int)((p.H + strips - 1) / strips);
    if (R < 16) R = 16;
  }
  if (R > p.H) R = p.H;
  a.R = R;
  a.nstrips = (p.H + R - 1) / R;
  a.nchunks = nbands;
  return a;
}

// Point the arguments at one step's buffers; `seed` is the step's seed before
// hashing (the call's seed plus the step index).
template <typename SF>
void tma_set_step(DevArgs<SF>& a, const char* src, char* dst, float* side_in, float* side_out, uint32_t seed) {
  const PackedLayout<SF> L = packed_layout<SF>(a.H, a.W);
  a.src_f = reinterpret_cast<const SF*>(src + L.off_f);
  a.src_g0 = reinterpret_cast<const float*>(src + L.off_g0);
  a.src_gi = reinterpret_cast<const SF*>(src + L.off_gi);
  a.dst_f = reinterpret_cast<SF*>(dst + L.off_f);
  a.dst_g0 = reinterpret_cast<float*>(dst + L.off_g0);
  a.dst_gi = reinterpret_cast<SF*>(dst + L.off_gi);
  a.side_in = side_in;
  a.side_out = side_out;
  a.seed = sr_hash(seed);
}

// One step over strips strip0 .. strip0 + nstrips - 1 of the lattice; `tm`:
// the tensor maps of the step's source buffer (tma_maps).
template <typename SF, int NT, int NS, bool SCALED, bool STOCH>
int launch_tma_strips(const DevArgs<SF>& a, const TmaMaps& tm, int strip0, int nstrips, cudaStream_t st) {
  using M = TmaSmem<SF, NT, NS>;
  if (tma_prepare_kernel<SF, NT, NS, SCALED, STOCH>() != cudaSuccess) return FD_ERR_CUDA;
  if (nstrips <= 0) return FD_OK;
  const unsigned blocks = (unsigned)(a.nchunks * nstrips);
  k_fused_tma<SF, NT, NS, SCALED, STOCH><<<blocks, NT, M::ALLOC, st>>>(a, a.nchunks, strip0, tm);
  return FD_OK;
}

template <typename SF, int NT, int NS, bool SCALED, bool STOCH>
int launch_fused_tma(const fd_params& p, const DevCoef& c, const uint16_t* mask, const double* inlet_ux, char* pa,
                     char* pb, float* sa, float* sb, int nsteps, int R, uint32_t seed, cudaStream_t st) {
  DevArgs<SF> a = tma_args<SF, NT, NS, SCALED, STOCH>(p, c, mask, inlet_ux, R);
  TmaMaps from_a, from_b;  // the source planes of even and of odd steps
  if (int r = tma_maps<SF, NT>(a, pa, from_a)) return r;
  if (int r = tma_maps<SF, NT>(a, pb, from_b)) return r;
  for (int s = 0; s < nsteps; ++s) {
    const bool even = s % 2 == 0;
    tma_set_step(a, even ? pa : pb, even ? pb : pa, even ? sa : sb, even ? sb : sa, seed + (uint32_t)s);
    if (int r = launch_tma_strips<SF, NT, NS, SCALED, STOCH>(a, even ? from_a : from_b, 0, a.nstrips, st)) return r;
  }
  return cudaGetLastError() == cudaSuccess ? FD_OK : FD_ERR_CUDA;
}

}  // namespace fd
