// Complex GEMM entry points of libgbblas: zgemm_/cblas_zgemm, cgemm_/
// cblas_cgemm, zgemm3m_/cblas_zgemm3m, cgemm3m_/cblas_cgemm3m and their
// device-pointer variants.
//
// Argument decoding follows interface/gemm.c compiled with COMPLEX (and with
// GEMM3M for the 3M names): op codes N = 0, T = 1, R = 2, C = 3
// (gemm.c:253-268, CBLAS ConjNoTrans/ConjTrans at gemm.c:395-411), the real
// GEMM's check order and xerbla positions (gemm.c:274-286), the row-major
// operand swap (gemm.c:423-471) and the quick return for m = 0 or n = 0
// (gemm.c:494).  alpha and beta are (re, im) pairs.
#include <string.h>

#include "gb_internal.h"
#include "operand.h"

namespace gb {

template <typename T>
int cgemm_device(int ta, int tb, int64_t m, int64_t n, int64_t k, const T *alpha, const T *A,
                 int64_t lda, const T *B, int64_t ldb, const T *beta, T *C, int64_t ldc,
                 int three_m, cudaStream_t s);

namespace {

inline int ztrans_code(char t) {
  t = upch(t);
  if (t == 'N') return 0;
  if (t == 'T') return 1;
  if (t == 'R') return 2;
  if (t == 'C') return 3;
  return -1;
}
inline int zcblas_trans_code(int t) {
  if (t == CblasNoTrans) return 0;
  if (t == CblasTrans) return 1;
  if (t == CblasConjNoTrans) return 2;
  if (t == CblasConjTrans) return 3;
  return -1;
}

template <typename T>
void cgemm_blocking(int ta, int tb, int64_t m, int64_t n, int64_t k, const T *alpha, const T *A,
                    int64_t lda, const T *B, int64_t ldb, const T *beta, T *C, int64_t ldc,
                    int three_m) {
  if (m == 0 || n == 0) return;
  if (ensure_init()) return;
  cudaStream_t s = stream();
  const size_t es = 2 * sizeof(T);
  const bool need_ab = k > 0 && !(alpha[0] == T(0) && alpha[1] == T(0));
  const bool beta_zero = beta[0] == T(0) && beta[1] == T(0);
  Operand a(A, (ta & 1) ? k : m, (ta & 1) ? m : k, lda, es);
  Operand b(B, (tb & 1) ? n : k, (tb & 1) ? k : n, ldb, es);
  Operand c(C, m, n, ldc, es);
  if (need_ab && (a.bind(true, s) || b.bind(true, s))) return;
  if (c.bind(!beta_zero, s)) return;
  if (cgemm_device<T>(ta, tb, m, n, k, alpha, a.d<T>(), a.dld, b.d<T>(), b.dld, beta, c.d<T>(),
                      c.dld, three_m, s))
    return;
  c.unbind(s);
  finish_blocking(s);
}

template <typename T>
void fortran_cgemm(const char *TRANSA, const char *TRANSB, const blasint *M, const blasint *N,
                   const blasint *K, const T *alpha, const T *A, const blasint *ldA, const T *B,
                   const blasint *ldB, const T *beta, T *C, const blasint *ldC, const char *name,
                   int three_m) {
  const int ta = ztrans_code(*TRANSA), tb = ztrans_code(*TRANSB);
  const int info = gemm_check(ta, tb, *M, *N, *K, *ldA, *ldB, *ldC);
  if (info) {
    call_xerbla(name, info);
    return;
  }
  cgemm_blocking<T>(ta, tb, *M, *N, *K, alpha, A, *ldA, B, *ldB, beta, C, *ldC, three_m);
}

template <typename T>
void cblas_cgemm_t(int order, int TransA, int TransB, blasint m, blasint n, blasint k,
                   const void *alpha, const void *a, blasint lda, const void *b, blasint ldb,
                   const void *beta, void *c, blasint ldc, const char *name, int three_m) {
  int info = -1, ta = -1, tb = -1;
  int64_t M = m, N = n;
  const T *pa = static_cast<const T *>(a), *pb = static_cast<const T *>(b);
  int64_t la = lda, lb = ldb;
  if (order == CblasColMajor) {
    ta = zcblas_trans_code(TransA);
    tb = zcblas_trans_code(TransB);
  } else if (order == CblasRowMajor) {
    M = n;
    N = m;
    pa = static_cast<const T *>(b);
    pb = static_cast<const T *>(a);
    la = ldb;
    lb = lda;
    ta = zcblas_trans_code(TransB);
    tb = zcblas_trans_code(TransA);
  }
  if (order == CblasColMajor || order == CblasRowMajor) {
    info = gemm_check(ta, tb, M, N, k, la, lb, ldc);
    if (info == 0) info = -1;
  }
  if (info >= 0) {
    call_xerbla(name, info);
    return;
  }
  cgemm_blocking<T>(ta, tb, M, N, k, static_cast<const T *>(alpha), pa, la, pb, lb,
                    static_cast<const T *>(beta), static_cast<T *>(c), ldc, three_m);
}

template <typename T>
int dev_cgemm(char transa, char transb, int64_t m, int64_t n, int64_t k, const T *alpha,
              const T *A, int64_t lda, const T *B, int64_t ldb, const T *beta, T *C, int64_t ldc,
              const char *name, int three_m) {
  const int ta = ztrans_code(transa), tb = ztrans_code(transb);
  const int info = gemm_check(ta, tb, m, n, k, lda, ldb, ldc);
  if (info) {
    call_xerbla(name, info);
    return GB_ERR_INVALID_VALUE;
  }
  const int st = ensure_init();
  if (st) return st;
  return cgemm_device<T>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, three_m,
                         stream());
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

void zgemm_(const char *TRANSA, const char *TRANSB, const blasint *M, const blasint *N,
            const blasint *K, const double *alpha, const double *A, const blasint *ldA,
            const double *B, const blasint *ldB, const double *beta, double *C,
            const blasint *ldC) {
  fortran_cgemm<double>(TRANSA, TRANSB, M, N, K, alpha, A, ldA, B, ldB, beta, C, ldC, "ZGEMM ",
                        0);
}

void cgemm_(const char *TRANSA, const char *TRANSB, const blasint *M, const blasint *N,
            const blasint *K, const float *alpha, const float *A, const blasint *ldA,
            const float *B, const blasint *ldB, const float *beta, float *C,
            const blasint *ldC) {
  fortran_cgemm<float>(TRANSA, TRANSB, M, N, K, alpha, A, ldA, B, ldB, beta, C, ldC, "CGEMM ",
                       0);
}

void zgemm3m_(const char *TRANSA, const char *TRANSB, const blasint *M, const blasint *N,
              const blasint *K, const double *alpha, const double *A, const blasint *ldA,
              const double *B, const blasint *ldB, const double *beta, double *C,
              const blasint *ldC) {
  fortran_cgemm<double>(TRANSA, TRANSB, M, N, K, alpha, A, ldA, B, ldB, beta, C, ldC,
                        "ZGEMM3M ", 1);
}

void cgemm3m_(const char *TRANSA, const char *TRANSB, const blasint *M, const blasint *N,
              const blasint *K, const float *alpha, const float *A, const blasint *ldA,
              const float *B, const blasint *ldB, const float *beta, float *C,
              const blasint *ldC) {
  fortran_cgemm<float>(TRANSA, TRANSB, M, N, K, alpha, A, ldA, B, ldB, beta, C, ldC,
                       "CGEMM3M ", 1);
}

void cblas_zgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA, enum CBLAS_TRANSPOSE TransB,
                 blasint M, blasint N, blasint K, const void *alpha, const void *A, blasint lda,
                 const void *B, blasint ldb, const void *beta, void *C, blasint ldc) {
  cblas_cgemm_t<double>(Order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc,
                        "ZGEMM ", 0);
}

void cblas_cgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA, enum CBLAS_TRANSPOSE TransB,
                 blasint M, blasint N, blasint K, const void *alpha, const void *A, blasint lda,
                 const void *B, blasint ldb, const void *beta, void *C, blasint ldc) {
  cblas_cgemm_t<float>(Order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc,
                       "CGEMM ", 0);
}

void cblas_zgemm3m(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA,
                   enum CBLAS_TRANSPOSE TransB, blasint M, blasint N, blasint K,
                   const void *alpha, const void *A, blasint lda, const void *B, blasint ldb,
                   const void *beta, void *C, blasint ldc) {
  cblas_cgemm_t<double>(Order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc,
                        "ZGEMM3M ", 1);
}

void cblas_cgemm3m(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA,
                   enum CBLAS_TRANSPOSE TransB, blasint M, blasint N, blasint K,
                   const void *alpha, const void *A, blasint lda, const void *B, blasint ldb,
                   const void *beta, void *C, blasint ldc) {
  cblas_cgemm_t<float>(Order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc,
                       "CGEMM3M ", 1);
}

int gb_zgemm_dev(char transa, char transb, int64_t m, int64_t n, int64_t k, const double *alpha,
                 const double *A, int64_t lda, const double *B, int64_t ldb, const double *beta,
                 double *C, int64_t ldc) {
  return dev_cgemm<double>(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                           "ZGEMM ", 0);
}

int gb_cgemm_dev(char transa, char transb, int64_t m, int64_t n, int64_t k, const float *alpha,
                 const float *A, int64_t lda, const float *B, int64_t ldb, const float *beta,
                 float *C, int64_t ldc) {
  return dev_cgemm<float>(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, "CGEMM ",
                          0);
}

int gb_zgemm3m_dev(char transa, char transb, int64_t m, int64_t n, int64_t k,
                   const double *alpha, const double *A, int64_t lda, const double *B,
                   int64_t ldb, const double *beta, double *C, int64_t ldc) {
  return dev_cgemm<double>(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                           "ZGEMM3M ", 1);
}

int gb_cgemm3m_dev(char transa, char transb, int64_t m, int64_t n, int64_t k, const float *alpha,
                   const float *A, int64_t lda, const float *B, int64_t ldb, const float *beta,
                   float *C, int64_t ldc) {
  return dev_cgemm<float>(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                          "CGEMM3M ", 1);
}

}  // extern "C"
