// Batched ensemble: many independent lattices (uneven sizes, geometries and
// parameters) advanced together by one persistent launch per iteration over a
// table of (instance, band, strip) tiles, with the iteration loop replayed
// from a CUDA graph.
#include <algorithm>
#include <vector>

#include "fd_fused_tma.cuh"
#include "fd_host.h"

struct fd_batch {
  int n = 0;
  fd_storage st{};
  int band = 128;     // cells per band = threads per CTA
  int rows = 32;      // rows per strip
  int parity = 0;     // 0: state in pop_a / side_a
  std::vector<fd_instance> inst;
  void* d_inst = nullptr;  // BatchInst<SF>[n]
  int4* d_tiles = nullptr;
  int ntiles = 0;
  int grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t graph_stream = nullptr;
  unsigned* d_ctl = nullptr;  // step and tile counters, two slots each (k_fused_tma_batch)
  unsigned* d_status = nullptr;  // per member: nonzero once a non-finite cell was met (quarantined)
};

namespace fd {
namespace {

template <typename SF>
DevArgs<SF> instance_args(const fd_instance& in, const fd_storage& st, int rows, bool swap, unsigned* status) {
  const fd_params& p = in.prm;
  const PackedLayout<SF> L = packed_layout<SF>(p.H, p.W);
  DevArgs<SF> a;
  a.c = make_dev_coef(p, st.f_scale_log2, st.g_scale_log2);
  a.H = p.H;
  a.W = p.W;
  a.variant = p.variant;
  // strips of equal height (within one row) at most `rows` high
  const int ns = (p.H + rows - 1) / rows;
  a.R = (p.H + ns - 1) / ns;
  a.nstrips = (p.H + a.R - 1) / a.R;
  a.nchunks = 0;
  a.P = L.P;
  a.pstride_f = L.pstride;
  a.mask = in.mask;
  a.inlet_ux = in.inlet_ux;
  char* src = (char*)(swap ? in.pop_b : in.pop_a);
  char* dst = (char*)(swap ? in.pop_a : in.pop_b);
  a.src_f = reinterpret_cast<const SF*>(src + L.off_f);
  a.src_g0 = reinterpret_cast<const float*>(src + L.off_g0);
  a.src_gi = reinterpret_cast<const SF*>(src + L.off_gi);
  a.dst_f = reinterpret_cast<SF*>(dst + L.off_f);
  a.dst_g0 = reinterpret_cast<float*>(dst + L.off_g0);
  a.dst_gi = reinterpret_cast<SF*>(dst + L.off_gi);
  a.side_in = (const float*)(swap ? in.side_b : in.side_a);
  a.side_out = (float*)(swap ? in.side_a : in.side_b);
  a.seed = in.seed;  // hashed with the batch step counter in the kernel
  a.status = status;
  return a;
}

template <typename SF, int NT, bool STOCH>
int prepare(fd_batch* b) {
  using M = TmaSmem<SF, NT, tma_ring_depth<SF>()>;
  auto kern = k_fused_tma_batch<SF, NT, tma_ring_depth<SF>(), false, STOCH>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, M::ALLOC) != cudaSuccess)
    return check_launch("fd_batch: shared-memory attribute");
  std::vector<BatchInst<SF>> hi(b->n);
  std::vector<int4> tiles;
  // members already flagged non-finite are not stepped any more: leave their
  // tiles out, so that the live members' tiles share the persistent grid
  std::vector<unsigned> flagged((size_t)b->n, 0u);
  if (cudaDeviceSynchronize() != cudaSuccess ||
      cudaMemcpy(flagged.data(), b->d_status, (size_t)b->n * sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess)
    return check_launch("fd_batch: member status");
  for (int i = 0; i < b->n; ++i) {
    hi[i].args[0] = instance_args<SF>(b->inst[i], b->st, b->rows, false, b->d_status + i);
    hi[i].args[1] = instance_args<SF>(b->inst[i], b->st, b->rows, true, b->d_status + i);
    if (int r = tma_maps<SF, NT>(hi[i].args[0], (const char*)b->inst[i].pop_a, hi[i].maps[0])) return r;
    if (int r = tma_maps<SF, NT>(hi[i].args[1], (const char*)b->inst[i].pop_b, hi[i].maps[1])) return r;
    const int nb = (b->inst[i].prm.W + NT - 1) / NT, ns = hi[i].args[0].nstrips;
    if (flagged[(size_t)i] != 0u) continue;
    for (int s = 0; s < ns; ++s)
      for (int bb = 0; bb < nb; ++bb) tiles.push_back(make_int4(i, bb, s, 0));
  }
  // largest first (rows of the tile's strip), ties in table order: the
  // kernel's counter then hands them out greedily
  auto strip_rows = [&](const int4& t) {
    const DevArgs<SF>& a = hi[t.x].args[0];
    const int y0 = t.z * a.R;
    return (y0 + a.R < a.H ? y0 + a.R : a.H) - y0;
  };
  std::stable_sort(tiles.begin(), tiles.end(),
                   [&](const int4& u, const int4& v) { return strip_rows(u) > strip_rows(v); });
  cudaFree(b->d_inst);
  cudaFree(b->d_tiles);
  b->d_inst = nullptr;
  b->d_tiles = nullptr;
  if (cudaMalloc(&b->d_inst, sizeof(BatchInst<SF>) * hi.size()) != cudaSuccess ||
      cudaMalloc(&b->d_tiles, sizeof(int4) * (tiles.empty() ? 1 : tiles.size())) != cudaSuccess)
    return check_launch("fd_batch: table allocation");
  if (cudaMemcpy(b->d_inst, hi.data(), sizeof(BatchInst<SF>) * hi.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      (!tiles.empty() &&
       cudaMemcpy(b->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice) != cudaSuccess))
    return check_launch("fd_batch: table upload");
  b->ntiles = (int)tiles.size();
  int per_sm = 1, dev = 0, sms = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, M::ALLOC);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  b->grid = per_sm * sms;
  if (b->grid > b->ntiles) b->grid = b->ntiles;
  if (b->grid < 1) b->grid = 1;
  return FD_OK;
}

template <typename SF, int NT, bool STOCH>
void launch_one(const fd_batch* b, int parity, cudaStream_t st) {
  using M = TmaSmem<SF, NT, tma_ring_depth<SF>()>;
  k_fused_tma_batch<SF, NT, tma_ring_depth<SF>(), false, STOCH><<<b->grid, NT, M::ALLOC, st>>>(
      (const BatchInst<SF>*)b->d_inst, b->d_tiles, b->ntiles, parity, b->d_ctl);
}

template <typename SF, bool STOCH>
int prepare_t(fd_batch* b) {
  switch (b->band) {
    case 64: return prepare<SF, 64, STOCH>(b);
    case 256: return prepare<SF, 256, STOCH>(b);
    default: return prepare<SF, 128, STOCH>(b);
  }
}

template <typename SF, bool STOCH>
void launch_t(const fd_batch* b, int parity, cudaStream_t st) {
  switch (b->band) {
    case 64: launch_one<SF, 64, STOCH>(b, parity, st); break;
    case 256: launch_one<SF, 256, STOCH>(b, parity, st); break;
    default: launch_one<SF, 128, STOCH>(b, parity, st); break;
  }
}

bool stochastic(const fd_batch* b) { return b->st.dtype != FD_F32 && b->st.rounding == FD_ROUND_STOCHASTIC; }

int prepare_any(fd_batch* b) {
  const bool sr = stochastic(b);
  switch (b->st.dtype) {
    case FD_F16: return sr ? prepare_t<__half, true>(b) : prepare_t<__half, false>(b);
    case FD_BF16: return sr ? prepare_t<__nv_bfloat16, true>(b) : prepare_t<__nv_bfloat16, false>(b);
    default: return prepare_t<float, false>(b);
  }
}

void launch_any(const fd_batch* b, int parity, cudaStream_t st) {
  const bool sr = stochastic(b);
  switch (b->st.dtype) {
    case FD_F16: sr ? launch_t<__half, true>(b, parity, st) : launch_t<__half, false>(b, parity, st); break;
    case FD_BF16:
      sr ? launch_t<__nv_bfloat16, true>(b, parity, st) : launch_t<__nv_bfloat16, false>(b, parity, st);
      break;
    default: launch_t<float, false>(b, parity, st); break;
  }
}

void drop_graph(fd_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->graph_stream = nullptr;
}

}  // namespace
}  // namespace fd

using namespace fd;

extern "C" {

int fd_batch_create(const fd_instance* inst, int n, const fd_storage* st, int rows_per_strip, int band_width,
                    fd_batch** out) {
  FD_REQUIRE(inst && n > 0 && st && out, FD_ERR_ARG, "fd_batch_create: bad arguments");
  FD_REQUIRE(st->dtype == FD_F32 || st->dtype == FD_F16 || st->dtype == FD_BF16, FD_ERR_DTYPE,
             "fd_batch_create: storage dtype %d", st->dtype);
  FD_REQUIRE(st->f_scale_log2 == 0 && st->g_scale_log2 == 0, FD_ERR_ARG,
             "fd_batch_create: scaled storage is not supported by the batched kernel");
  FD_REQUIRE(st->rounding == FD_ROUND_NEAREST || st->rounding == FD_ROUND_STOCHASTIC, FD_ERR_ARG,
             "fd_batch_create: storage rounding %d", st->rounding);
  FD_REQUIRE(band_width == 64 || band_width == 128 || band_width == 256, FD_ERR_ARG,
             "fd_batch_create: band width must be 64, 128 or 256");
  FD_REQUIRE(rows_per_strip >= 1, FD_ERR_ARG, "fd_batch_create: rows per strip must be positive");
  for (int i = 0; i < n; ++i) {
    if (int r = check_params(&inst[i].prm)) return r;
    FD_REQUIRE(inst[i].prm.variant != FD_VARIANT_PERIODIC_XY, FD_ERR_SHAPE,
               "fd_batch_create: instance %d uses the periodic-xy variant (reference-order kernels only)", i);
    FD_REQUIRE(inst[i].prm.W % 8 == 0, FD_ERR_SHAPE, "fd_batch_create: instance %d width %d is not a multiple of 8",
               i, inst[i].prm.W);
    FD_REQUIRE(inst[i].mask && inst[i].inlet_ux && inst[i].pop_a && inst[i].pop_b && inst[i].side_a &&
                   inst[i].side_b,
               FD_ERR_ARG, "fd_batch_create: instance %d has a NULL pointer", i);
    FD_REQUIRE(((uintptr_t)inst[i].pop_a | (uintptr_t)inst[i].pop_b) % 256 == 0 && (uintptr_t)inst[i].mask % 16 == 0,
               FD_ERR_ARG, "fd_batch_create: instance %d buffers are not aligned", i);
  }
  fd_batch* b = new fd_batch;
  b->n = n;
  b->st = *st;
  b->band = band_width;
  b->rows = rows_per_strip;
  b->inst.assign(inst, inst + n);
  if (cudaMalloc(&b->d_ctl, 4 * sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(b->d_ctl, 0, 4 * sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(&b->d_status, (size_t)n * sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(b->d_status, 0, (size_t)n * sizeof(unsigned)) != cudaSuccess) {
    const int r = check_launch("fd_batch_create: step counter");
    fd_batch_destroy(b);
    return r;
  }
  if (int r = prepare_any(b)) {
    fd_batch_destroy(b);
    return r;
  }
  *out = b;
  return FD_OK;
}

int fd_batch_configure(fd_batch* b, int rows_per_strip, int band_width) {
  FD_REQUIRE(b != nullptr, FD_ERR_ARG, "fd_batch_configure: NULL batch");
  FD_REQUIRE(band_width == 64 || band_width == 128 || band_width == 256, FD_ERR_ARG,
             "fd_batch_configure: band width must be 64, 128 or 256");
  FD_REQUIRE(rows_per_strip >= 1, FD_ERR_ARG, "fd_batch_configure: rows per strip must be positive");
  drop_graph(b);
  b->band = band_width;
  b->rows = rows_per_strip;
  return prepare_any(b);
}

int fd_batch_step(fd_batch* b, int nsteps, int use_graph, void* stream) {
  FD_REQUIRE(b != nullptr && nsteps >= 0, FD_ERR_ARG, "fd_batch_step: bad arguments");
  cudaStream_t st = as_stream(stream);
  FD_REQUIRE(!use_graph || st != nullptr, FD_ERR_ARG, "fd_batch_step: graph replay needs a non-default stream");
  int left = nsteps;
  if (use_graph && left >= 2) {
    if (b->parity == 1) {  // the graph starts at parity 0
      launch_any(b, 1, st);
      b->parity = 0;
      --left;
    }
    if (b->exec == nullptr || b->graph_stream != st) {
      drop_graph(b);
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return check_launch("fd_batch_step: begin capture");
      launch_any(b, 0, st);
      launch_any(b, 1, st);
      if (cudaStreamEndCapture(st, &b->graph) != cudaSuccess) return check_launch("fd_batch_step: end capture");
      if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) return check_launch("fd_batch_step: instantiate");
      b->graph_stream = st;
    }
    for (; left >= 2; left -= 2)
      if (cudaGraphLaunch(b->exec, st) != cudaSuccess) return check_launch("fd_batch_step: graph launch");
  }
  for (; left > 0; --left) {
    launch_any(b, b->parity, st);
    b->parity ^= 1;
  }
  return check_launch("fd_batch_step");
}

int fd_batch_parity(const fd_batch* b) { return b ? b->parity : -1; }

int fd_batch_member_status(fd_batch* b, uint32_t* out, int clear) {
  FD_REQUIRE(b != nullptr && out != nullptr, FD_ERR_ARG, "fd_batch_member_status: NULL pointer");
  if (cudaDeviceSynchronize() != cudaSuccess ||
      cudaMemcpy(out, b->d_status, (size_t)b->n * sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess)
    return check_launch("fd_batch_member_status");
  if (clear && cudaMemset(b->d_status, 0, (size_t)b->n * sizeof(unsigned)) != cudaSuccess)
    return check_launch("fd_batch_member_status: clear");
  for (int i = 0; i < b->n; ++i)
    FD_REQUIRE(out[i] == 0, FD_ERR_NONFINITE, "fd_batch_member_status: member %d met a non-finite cell", i);
  return FD_OK;
}

int fd_batch_tiles(const fd_batch* b) { return b ? b->ntiles : -1; }

int fd_batch_grid(const fd_batch* b) { return b ? b->grid : -1; }

int fd_batch_destroy(fd_batch* b) {
  if (!b) return FD_OK;
  drop_graph(b);
  cudaFree(b->d_inst);
  cudaFree(b->d_tiles);
  cudaFree(b->d_ctl);
  cudaFree(b->d_status);
  delete b;
  return FD_OK;
}

}  // extern "C"

namespace fd {

// This unit's copy of the device error word (fd_fused_dev.cuh), which the
// batched kernel latches; fd_device_status() combines it with the others.
int batch_device_error(unsigned* out, bool clear) { return device_error_word(out, clear); }

// The failure path of the bounded wait, on this unit's error word: one thread
// waits on an mbarrier that nothing arrives on and gives up after `polls`.
__global__ void k_selftest_wait_timeout_batch(unsigned polls) {
  __shared__ uint64_t bar;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  mbar_wait(&bar, 0u, polls);
}

int batch_selftest_wait_timeout(unsigned polls, cudaStream_t s) {
  k_selftest_wait_timeout_batch<<<1, 1, 0, s>>>(polls);
  return FD_OK;
}

}  // namespace fd
