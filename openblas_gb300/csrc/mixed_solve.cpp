// Mixed-precision DGESV (placeholder until the FP32-LU + refinement path lands).
#include "gb_internal.h"
#include "operand.h"

extern "C" int dsgesv_(const blasint *, const blasint *, double *, const blasint *, blasint *,
                       const double *, const blasint *, double *, const blasint *, double *,
                       float *, blasint *, blasint *Info) {
  *Info = 0;
  return gb::set_error(GB_ERR_UNSUPPORTED, "dsgesv not built");
}
extern "C" int gb_dsgesv_dev(int64_t, int64_t, const double *, int64_t, int *, const double *,
                             int64_t, double *, int64_t, int *, int *) {
  return gb::set_error(GB_ERR_UNSUPPORTED, "dsgesv not built");
}
