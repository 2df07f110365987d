// FP64 diagnostics of a lattice state: colour masses, saturation, finger tip
// and breakthrough.
//
// The reference defines none of these (it only plots psi); they are the
// quantities the invasion is judged by:
//   mass_r = sum over fluid cells of rho (1 + psi) / 2   (invading fluid)
//   mass_b = sum over fluid cells of rho (1 - psi) / 2   (defending fluid)
//   invaded = number of fluid cells with psi > 0, saturation = invaded / fluid
//   tip_x  = largest x of a fluid cell with psi > 0 (-1 if none)
//   breakthrough = some fluid cell with x >= W-5 has psi > 0
// (the outlet's Zou-He rule for g pins psi = -1 on column W-1, and the
// mobility term pulls the columns next to it towards -1, so invading fluid
// arriving at the outlet is seen in the last five columns, never in the last)
// rho = sum f_i and psi = sum g_i are read from the stored populations: the
// collision conserves both at every cell (sum of the forcing terms is zero,
// fingering_periodic.py:194-199), so pre- and post-collision states give the
// same values.  Sums are accumulated in FP64 in a fixed order (per-block
// partials, then one block over the partials), so the result is reproducible.
#include "fd_fused_dev.cuh"
#include "fd_host.h"

namespace fd {
namespace {

constexpr int kDiagThreads = 256;
constexpr int kDiagBlocks = 1024;  // partials per reduction (fixed -> deterministic)
constexpr int kOutletBand = 5;     // breakthrough columns: x >= W - kOutletBand

struct Partial {
  double mass_r, mass_b;
  long long invaded, fluid;
  int tip_x, breakthrough;
};

template <typename T>
struct RefLayout {  // (18, H, W) of T: f planes then g planes
  const T* p;
  size_t P;
  __device__ void cell(size_t q, double& rho, double& psi) const {
    double r = 0.0, s = 0.0;
#pragma unroll
    for (int i = 0; i < 9; ++i) r += (double)p[i * P + q];
#pragma unroll
    for (int i = 0; i < 9; ++i) s += (double)p[(9 + i) * P + q];
    rho = r;
    psi = s;
  }
};

template <typename SF>
struct PackedView {  // packed deviation layout
  const SF* f;
  const float* g0;
  const SF* gi;
  size_t ps;
  float inv_sf, inv_sg;
  __device__ void cell(size_t q, double& rho, double& psi) const {
    double r = 1.0, s = (double)g0[q];
#pragma unroll
    for (int i = 0; i < 9; ++i) r += (double)(to_f<SF>(f[i * ps + q]) * inv_sf);
#pragma unroll
    for (int i = 0; i < 8; ++i) s += (double)(to_f<SF>(gi[i * ps + q]) * inv_sg);
    rho = r;
    psi = s;
  }
};

template <typename View>
__global__ void k_diag_partial(View v, const uint16_t* __restrict__ mask, int H, int W, Partial* __restrict__ out) {
  __shared__ double s_r[kDiagThreads], s_b[kDiagThreads];
  __shared__ long long s_n[kDiagThreads], s_f[kDiagThreads];
  __shared__ int s_tip[kDiagThreads], s_bt[kDiagThreads];
  const size_t P = (size_t)H * W;
  const size_t per = (P + gridDim.x - 1) / gridDim.x;
  const size_t lo = (size_t)blockIdx.x * per, hi = min(P, lo + per);
  double mr = 0.0, mb = 0.0;
  long long n = 0, nf = 0;
  int tip = -1, bt = 0;
  for (size_t q = lo + threadIdx.x; q < hi; q += blockDim.x) {
    if (mask[q] & SOLID) continue;
    double rho, psi;
    v.cell(q, rho, psi);
    mr += rho * (1.0 + psi) * 0.5;
    mb += rho * (1.0 - psi) * 0.5;
    ++nf;
    if (psi > 0.0) {
      ++n;
      const int x = (int)(q % W);
      tip = max(tip, x);
      if (x >= W - kOutletBand) bt = 1;
    }
  }
  const int t = threadIdx.x;
  s_r[t] = mr; s_b[t] = mb; s_n[t] = n; s_f[t] = nf; s_tip[t] = tip; s_bt[t] = bt;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      s_r[t] += s_r[t + w]; s_b[t] += s_b[t + w]; s_n[t] += s_n[t + w]; s_f[t] += s_f[t + w];
      s_tip[t] = max(s_tip[t], s_tip[t + w]); s_bt[t] |= s_bt[t + w];
    }
    __syncthreads();
  }
  if (t == 0) out[blockIdx.x] = Partial{s_r[0], s_b[0], s_n[0], s_f[0], s_tip[0], s_bt[0]};
}

__global__ void k_diag_final(const Partial* __restrict__ in, int n, fd_diag* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Partial a{0.0, 0.0, 0, 0, -1, 0};
  for (int i = 0; i < n; ++i) {  // fixed order
    a.mass_r += in[i].mass_r; a.mass_b += in[i].mass_b;
    a.invaded += in[i].invaded; a.fluid += in[i].fluid;
    a.tip_x = max(a.tip_x, in[i].tip_x); a.breakthrough |= in[i].breakthrough;
  }
  out->mass_r = a.mass_r;
  out->mass_b = a.mass_b;
  out->invaded = a.invaded;
  out->fluid = a.fluid;
  out->saturation = a.fluid ? (double)a.invaded / (double)a.fluid : 0.0;
  out->tip_x = a.tip_x;
  out->breakthrough = a.breakthrough;
}

template <typename View>
int launch_diag(View v, const uint16_t* mask, int H, int W, void* scratch, fd_diag* out, cudaStream_t st) {
  k_diag_partial<View><<<kDiagBlocks, kDiagThreads, 0, st>>>(v, mask, H, W, (Partial*)scratch);
  k_diag_final<<<1, 32, 0, st>>>((const Partial*)scratch, kDiagBlocks, out);
  return check_launch("fd_diagnostics");
}

}  // namespace
}  // namespace fd

using namespace fd;

extern "C" {

size_t fd_diag_scratch_bytes(void) { return sizeof(Partial) * kDiagBlocks; }

int fd_diagnostics(const fd_params* prm, int dtype, const fd_storage* st, const void* pop, const uint16_t* mask,
                   void* scratch, fd_diag* out, void* stream) {
  if (int r = check_params(prm)) return r;
  FD_REQUIRE(pop && mask && scratch && out, FD_ERR_ARG, "fd_diagnostics: NULL pointer");
  cudaStream_t s = as_stream(stream);
  const int H = prm->H, W = prm->W;
  const size_t P = (size_t)H * W;
  if (st == nullptr) {
    FD_REQUIRE(dtype == FD_F64 || dtype == FD_F32, FD_ERR_DTYPE, "fd_diagnostics: dtype %d", dtype);
    if (dtype == FD_F64) return launch_diag(RefLayout<double>{(const double*)pop, P}, mask, H, W, scratch, out, s);
    return launch_diag(RefLayout<float>{(const float*)pop, P}, mask, H, W, scratch, out, s);
  }
  FD_REQUIRE(st->dtype == FD_F32 || st->dtype == FD_F16 || st->dtype == FD_BF16, FD_ERR_DTYPE,
             "fd_diagnostics: packed storage dtype %d", st->dtype);
  const char* b = (const char*)pop;
  const float isf = ldexpf(1.0f, -st->f_scale_log2), isg = ldexpf(1.0f, -st->g_scale_log2);
  switch (st->dtype) {
    case FD_F16: {
      const PackedLayout<__half> L = packed_layout<__half>(H, W);
      return launch_diag(PackedView<__half>{(const __half*)(b + L.off_f), (const float*)(b + L.off_g0),
                                            (const __half*)(b + L.off_gi), L.pstride, isf, isg},
                         mask, H, W, scratch, out, s);
    }
    case FD_BF16: {
      const PackedLayout<__nv_bfloat16> L = packed_layout<__nv_bfloat16>(H, W);
      return launch_diag(PackedView<__nv_bfloat16>{(const __nv_bfloat16*)(b + L.off_f), (const float*)(b + L.off_g0),
                                                   (const __nv_bfloat16*)(b + L.off_gi), L.pstride, isf, isg},
                         mask, H, W, scratch, out, s);
    }
    default: {
      const PackedLayout<float> L = packed_layout<float>(H, W);
      return launch_diag(PackedView<float>{(const float*)(b + L.off_f), (const float*)(b + L.off_g0),
                                           (const float*)(b + L.off_gi), L.pstride, 1.0f, 1.0f},
                         mask, H, W, scratch, out, s);
    }
  }
}

}  // extern "C"
