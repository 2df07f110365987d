// The host-resident step (fd_fused_step_packed_host): the packed state lives
// in host memory, as the reference's numpy arrays do, and one call uploads it,
// advances it and downloads the result.  The transfers dominate (a step of
// the 4096 x 2048 FP32 lattice moves 604 MB each way over the host link and
// computes for 0.23 ms), so the call pipelines them over chunks of rows:
//
//   upload stream   : chunk 0, 1, ..., K-1 host -> device
//   caller's stream : chunk c of the step once rows c-2 .. c+1 have landed
//                     (order 1 .. K-2, then K-1 and 0, whose neighbours wrap)
//   download stream : chunk c device -> host once it is computed
//
// so the two copy directions run at the same time and the kernel runs under
// them.  The download stream is the slower one and cannot start before chunks
// 0..2 have landed and chunk 1 is computed, so the first chunks are small
// (1, 1, 2, 4 strips) and the rest about 1/16 of the lattice.  A chunk is a
// whole number of strips of the staged kernel; every cell is computed exactly
// as by fd_fused_step_packed (strips only schedule the work), so the results
// are identical.
#include <algorithm>
#include <mutex>
#include <vector>

#include "fd_fused_dev.cuh"
#include "fd_host.h"
#include "fd_host_plan.h"

namespace fd {

int fused_tma_strips(const fd_params& p, const fd_storage& st, const DevCoef& c, const uint16_t* mask,
                     const double* inlet_ux, const void* src, void* dst, const void* side_in, void* side_out, int R,
                     int strip0, int nstrips, uint32_t seed, cudaStream_t s);

namespace {

// Streams and events of the pipeline, one set per device, created on first
// use and kept for the life of the process.  Calls on one device serialise on
// the mutex while they enqueue (a later record of an event does not affect
// waits enqueued before it, so the sets can be reused at once).
struct Pipe {
  std::mutex mu;
  bool ready = false;
  cudaStream_t up = nullptr, down = nullptr;
  cudaEvent_t fork = nullptr, up_done = nullptr, done_down = nullptr;
  std::vector<cudaEvent_t> ev_up, ev_comp;
};

Pipe g_pipes[64];

int pipe_init(Pipe& p) {
  if (p.ready) return FD_OK;
  auto ev = [](cudaEvent_t* e) { return cudaEventCreateWithFlags(e, cudaEventDisableTiming); };
  if (cudaStreamCreateWithFlags(&p.up, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&p.down, cudaStreamNonBlocking) != cudaSuccess || ev(&p.fork) != cudaSuccess ||
      ev(&p.up_done) != cudaSuccess || ev(&p.done_down) != cudaSuccess)
    return check_launch("fd_fused_step_packed_host: stream/event creation");
  p.ev_up.resize(kMaxChunks);
  p.ev_comp.resize(kMaxChunks);
  for (int i = 0; i < kMaxChunks; ++i)
    if (ev(&p.ev_up[i]) != cudaSuccess || ev(&p.ev_comp[i]) != cudaSuccess)
      return check_launch("fd_fused_step_packed_host: event creation");
  p.ready = true;
  return FD_OK;
}

// Plane geometry of a packed buffer: 9 f planes of `es` bytes per cell, the
// FP32 g_0 plane, 8 g_i planes of `es` bytes; every plane starts on a 256-byte
// boundary (fd_fused_dev.cuh).
struct Planes {
  size_t es, bf, bg, off_g0, off_gi;
};

Planes planes_of(const fd_params& p, int dtype) {
  Planes q;
  const size_t P = (size_t)p.H * p.W;
  q.es = dtype == FD_F32 ? 4 : 2;
  q.bf = plane_bytes(P, q.es);
  q.bg = plane_bytes(P, 4);
  q.off_g0 = 9 * q.bf;
  q.off_gi = q.off_g0 + q.bg;
  return q;
}

// Copy rows r0 .. r1-1 of every plane between two packed buffers.
cudaError_t copy_rows(const Planes& q, int W, int r0, int r1, char* dst, const char* src, cudaMemcpyKind kind,
                      cudaStream_t s) {
  const size_t n = (size_t)(r1 - r0) * W;
  const size_t of = (size_t)r0 * W * q.es, og = (size_t)r0 * W * 4;
  if (q.es == 4)  // 18 planes of one size: one strided copy
    return cudaMemcpy2DAsync(dst + of, q.bf, src + of, q.bf, n * 4, 18, kind, s);
  cudaError_t e = cudaMemcpy2DAsync(dst + of, q.bf, src + of, q.bf, n * q.es, 9, kind, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dst + q.off_g0 + og, src + q.off_g0 + og, n * 4, kind, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(dst + q.off_gi + of, q.bf, src + q.off_gi + of, q.bf, n * q.es, 8, kind, s);
  return e;
}

// Enqueue the uploads, the iterations and the downloads (after the fork).
int host_pipeline(Pipe& pipe, const fd_params& prm, const fd_storage& st, const DevCoef& coef, const uint16_t* mask,
                  const double* inlet_ux, const Planes& q, const HostPlan& plan, int nsteps, const char* hin,
                  char* hout, char* pa, char* pb, float* sa, float* sb, cudaStream_t s);

}  // namespace
}  // namespace fd

extern "C" int fd_fused_step_packed_host(const fd_params* prm, const fd_storage* st, const uint16_t* mask,
                                         const double* inlet_ux, const void* host_in, void* host_out, void* pop_a,
                                         void* pop_b, void* side_a, void* side_b, int nsteps, int chunk_rows,
                                         void* stream) {
  using namespace fd;
  if (int r = check_params(prm)) return r;
  const size_t nbytes = fd_packed_bytes(prm->H, prm->W, st);  // validates the storage descriptor
  if (nbytes == 0) return FD_ERR_ARG;
  FD_REQUIRE(prm->variant != FD_VARIANT_PERIODIC_XY, FD_ERR_SHAPE,
             "fd_fused_step_packed_host: the periodic-xy variant has no packed step");
  FD_REQUIRE(host_in && host_out && mask && inlet_ux && pop_a && pop_b && side_a && side_b, FD_ERR_ARG,
             "fd_fused_step_packed_host: NULL pointer");
  FD_REQUIRE(pop_a != pop_b && side_a != side_b, FD_ERR_ARG,
             "fd_fused_step_packed_host: ping-pong buffers must differ");
  FD_REQUIRE(nsteps >= 1, FD_ERR_ARG, "fd_fused_step_packed_host: nsteps must be >= 1");
  FD_REQUIRE(prm->W % 8 == 0 && prm->W >= 8 && prm->H >= 3, FD_ERR_SHAPE,
             "fd_fused_step_packed_host: W must be a multiple of 8, H >= 3 (got %dx%d)", prm->H, prm->W);
  FD_REQUIRE(((uintptr_t)pop_a | (uintptr_t)pop_b) % 256 == 0, FD_ERR_ARG,
             "fd_fused_step_packed_host: population buffers must be 256-byte aligned");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("fd_fused_step_packed_host");
  FD_REQUIRE(dev >= 0 && dev < 64, FD_ERR_ARG, "fd_fused_step_packed_host: device ordinal %d", dev);

  const HostPlan plan = host_plan(prm->H, chunk_rows);

  const Planes q = planes_of(*prm, st->dtype);
  const DevCoef coef = make_dev_coef(*prm, st->f_scale_log2, st->g_scale_log2);
  cudaStream_t s = as_stream(stream);
  Pipe& pipe = g_pipes[dev];
  std::lock_guard<std::mutex> lock(pipe.mu);
  if (int r = pipe_init(pipe)) return r;

  char* pa = (char*)pop_a;
  char* pb = (char*)pop_b;
  float* sa = (float*)side_a;
  float* sb = (float*)side_b;
  const char* hin = (const char*)host_in;
  char* hout = (char*)host_out;

  // fork: the copies start after the work already on the caller's stream
  if (cudaEventRecord(pipe.fork, s) != cudaSuccess || cudaStreamWaitEvent(pipe.up, pipe.fork, 0) != cudaSuccess ||
      cudaStreamWaitEvent(pipe.down, pipe.fork, 0) != cudaSuccess)
    return check_launch("fd_fused_step_packed_host: fork");
  const int r = host_pipeline(pipe, *prm, *st, coef, mask, inlet_ux, q, plan, nsteps, hin, hout, pa, pb, sa, sb, s);
  // join, also after a failure: the caller's stream continues after the
  // copies already issued on both internal streams
  const bool joined = cudaEventRecord(pipe.up_done, pipe.up) == cudaSuccess &&
                      cudaEventRecord(pipe.done_down, pipe.down) == cudaSuccess &&
                      cudaStreamWaitEvent(s, pipe.up_done, 0) == cudaSuccess &&
                      cudaStreamWaitEvent(s, pipe.done_down, 0) == cudaSuccess;
  if (r != FD_OK) return r;
  if (!joined) return check_launch("fd_fused_step_packed_host: join");
  return check_launch("fd_fused_step_packed_host");
}

namespace fd {
namespace {

int host_pipeline(Pipe& pipe, const fd_params& prm, const fd_storage& st, const DevCoef& coef, const uint16_t* mask,
                  const double* inlet_ux, const Planes& q, const HostPlan& plan, int nsteps, const char* hin,
                  char* hout, char* pa, char* pb, float* sa, float* sb, cudaStream_t s) {
  const std::vector<int>& cb = plan.cb;
  const int K = (int)cb.size() - 1, H = prm.H, W = prm.W, R = plan.R, nstrips = plan.nstrips;
  auto rows_of = [&](int c, int& r0, int& r1) {
    r0 = cb[c] * R;
    r1 = std::min(cb[c + 1] * R, H);
  };
  for (int c = 0; c < K; ++c) {
    int r0, r1;
    rows_of(c, r0, r1);
    if (copy_rows(q, W, r0, r1, pa, hin, cudaMemcpyHostToDevice, pipe.up) != cudaSuccess ||
        cudaEventRecord(pipe.ev_up[c], pipe.up) != cudaSuccess)
      return check_launch("fd_fused_step_packed_host: upload");
  }
  for (int step = 0; step < nsteps; ++step) {
    const bool even = step % 2 == 0;
    char* src = even ? pa : pb;
    char* dst = even ? pb : pa;
    float* sin = even ? sa : sb;
    float* sout = even ? sb : sa;
    const uint32_t seed = st.seed + (uint32_t)step;
    const bool first = step == 0, last = step == nsteps - 1;
    if (!first && !last) {  // a middle step: one launch over the whole lattice
      if (int r = fused_tma_strips(prm, st, coef, mask, inlet_ux, src, dst, sin, sout, R, 0, nstrips, seed, s))
        return r;
      continue;
    }
    for (int c : plan.order) {
      if (first) {
        if (cudaStreamWaitEvent(s, pipe.ev_up[plan.need[c]], 0) != cudaSuccess)
          return check_launch("fd_fused_step_packed_host: wait for upload");
      }
      const int s0 = cb[c], ns = cb[c + 1] - cb[c];
      if (int r = fused_tma_strips(prm, st, coef, mask, inlet_ux, src, dst, sin, sout, R, s0, ns, seed, s))
        return r;
      if (last) {
        int r0, r1;
        rows_of(c, r0, r1);
        if (cudaEventRecord(pipe.ev_comp[c], s) != cudaSuccess ||
            cudaStreamWaitEvent(pipe.down, pipe.ev_comp[c], 0) != cudaSuccess ||
            copy_rows(q, W, r0, r1, hout, dst, cudaMemcpyDeviceToHost, pipe.down) != cudaSuccess)
          return check_launch("fd_fused_step_packed_host: download");
      }
    }
  }
  return FD_OK;
}

}  // namespace
}  // namespace fd
