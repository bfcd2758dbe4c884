// Host side of the TMA loads: 2-D tensor maps over K-contiguous bf16
// operand slices (rows x kpad, K innermost, 128-byte swizzle), encoded
// through the driver entry point cuTensorMapEncodeTiled (resolved once at
// run time, so the library links against the CUDA runtime only).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_internal.h"

namespace gb {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Resolved once per process (thread-safe static initialisation); null when
// the driver does not provide it.
inline EncodeTiledFn tma_encode_fn() {
  static const EncodeTiledFn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<EncodeTiledFn>(p);
    cudaGetLastError();
    return static_cast<EncodeTiledFn>(nullptr);
  }();
  return fn;
}

// Map over `rows` x `kpad` bf16 at `base` (row stride kpad * 2 bytes, a
// multiple of 128), box of box_k (64 for the 128-byte swizzle) x box_rows.
inline int make_bf16_kmajor_map(CUtensorMap *map, void *base, int64_t rows, int64_t kpad,
                                int box_k, int box_rows) {
  EncodeTiledFn fn = tma_encode_fn();
  if (!fn) return set_error(GB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
  cuuint32_t box[2] = {(cuuint32_t)box_k, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(GB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return GB_SUCCESS;
}

}  // namespace gb
