// Grouped uneven GEMM batch (cblas_dgemm_batch), per-problem form.
#include <vector>

#include "gb_internal.h"
#include "operand.h"

namespace gb {

int dgemm_batch_loop(int order, const int *ta, const int *tb, const blasint *m,
                     const blasint *n, const blasint *k, const double *alpha, const double **A,
                     const blasint *lda, const double **B, const blasint *ldb,
                     const double *beta, double **C, const blasint *ldc, blasint group_count,
                     const blasint *group_size) {
  int st = ensure_init();
  if (st) return st;
  cudaStream_t s = stream();
  int64_t idx = 0;
  for (blasint g = 0; g < group_count; ++g) {
    const bool row = order == CblasRowMajor;
    const int64_t M = row ? n[g] : m[g], N = row ? m[g] : n[g], K = k[g];
    for (blasint t = 0; t < group_size[g]; ++t, ++idx) {
      const double *pa = row ? B[idx] : A[idx];
      const double *pb = row ? A[idx] : B[idx];
      const int64_t la = row ? ldb[g] : lda[g], lb = row ? lda[g] : ldb[g];
      if (M == 0 || N == 0) continue;
      const bool need_ab = K > 0 && alpha[g] != 0.0;
      Operand a(pa, ta[g] ? K : M, ta[g] ? M : K, la, 8);
      Operand b(pb, tb[g] ? N : K, tb[g] ? K : N, lb, 8);
      Operand c(C[idx], M, N, ldc[g], 8);
      if (need_ab && ((st = a.bind(true, s)) || (st = b.bind(true, s)))) return st;
      if ((st = c.bind(beta[g] != 0.0, s))) return st;
      if (!need_ab)
        launch_dgemm_beta(M, N, beta[g], c.d<double>(), c.dld, s);
      else
        launch_dgemm_fp64(ta[g], tb[g], M, N, K, alpha[g], a.d<double>(), a.dld, b.d<double>(),
                          b.dld, beta[g], c.d<double>(), c.dld, s);
      if ((st = c.unbind(s))) return st;
    }
  }
  return finish_blocking(s);
}

int gb_dgemm_batch_grouped(int order, const int *ta, const int *tb, const blasint *m,
                           const blasint *n, const blasint *k, const double *alpha,
                           const double **A, const blasint *lda, const double **B,
                           const blasint *ldb, const double *beta, double **C,
                           const blasint *ldc, blasint group_count, const blasint *group_size) {
  return dgemm_batch_loop(order, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                          group_count, group_size);
}

}  // namespace gb
