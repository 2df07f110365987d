// Tensor maps (TMA descriptors) of the packed population planes, encoded on
// the host.  cuTensorMapEncodeTiled is taken from the driver through the
// runtime's entry-point query, so the library does not link libcuda.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "fd_host.h"

namespace fd {

// The source planes of one step for the staged kernel: the nine f planes, the
// eight g_i planes and the FP32 g_0 plane of a packed buffer, each a 3-D
// tensor (x, row, plane) whose box is one band row of every plane.
struct alignas(128) TmaMaps {
  CUtensorMap f, gi, g0;
};

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_tiled_fn() {
  static const EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (EncodeTiledFn) nullptr;
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// 3-D map over `planes` planes of H x W elements of `es` (2 or 4) bytes,
// planes `plane_bytes` apart, box = `box_x` consecutive cells of one row of
// every plane (landing in shared memory as `planes` rows of box_x * es bytes).
// Cells outside [0, W) read as zero.
inline int encode_plane_rows(CUtensorMap* m, const void* base, int es, int W, int H, int planes, size_t plane_bytes,
                             int box_x) {
  FD_REQUIRE(((uintptr_t)base % 16) == 0 && ((size_t)W * es) % 16 == 0 && plane_bytes % 16 == 0 &&
                 ((size_t)box_x * es) % 16 == 0 && box_x <= 256 && planes <= 256 &&
                 plane_bytes >= (size_t)W * H * es,
             FD_ERR_ARG, "tensor map: unaligned base, stride or box (W=%d, es=%d, box %d)", W, es, box_x);
  const EncodeTiledFn fn = encode_tiled_fn();
  FD_REQUIRE(fn != nullptr, FD_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint64_t dim[3] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)planes};
  const cuuint64_t stride[2] = {(cuuint64_t)W * es, (cuuint64_t)plane_bytes};
  const cuuint32_t box[3] = {(cuuint32_t)box_x, 1u, (cuuint32_t)planes};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  const CUresult r = fn(m, es == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 3,
                        const_cast<void*>(base), dim, stride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  FD_REQUIRE(r == CUDA_SUCCESS, FD_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return FD_OK;
}

}  // namespace fd
