// Emulated FP64 GEMM (placeholder until the tensor-core path lands).
#include "gb_internal.h"
namespace gb {
int dgemm_emulated(int, int, int64_t, int64_t, int64_t, double, const double *, int64_t,
                   const double *, int64_t, double, double *, int64_t, int, cudaStream_t) {
  return set_error(GB_ERR_UNSUPPORTED, "emulated DGEMM not built");
}
}  // namespace gb
