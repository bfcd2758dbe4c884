/*
 * oracle.h -- CPU restatement of OpenBLAS's level-3 + blocked-LAPACK hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library gives the results the product is
 * tested against: only the tests, the smoke check and the CPU-baseline leg of
 * bench.py may load it.  The product
 * (libgbblas.so) never links, loads or calls it.
 *
 * Every routine restates the reference algorithm it cites (paths are relative
 * to the OpenBLAS source tree, version 0.3.28.dev).  All matrices are
 * column-major; ipiv is 1-based, as in the Fortran ABI.  Parity of this
 * restatement is pinned against golden vectors produced by an OpenBLAS build
 * (tests/golden/gen_golden.py) -- see the tests.
 */
#ifndef GB_ORACLE_H
#define GB_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Number of OpenMP threads the oracle may use (0 = all available). */
void orc_set_threads(int n);
int orc_get_threads(void);

/* C <- alpha*op(A)*op(B) + beta*C.  beta==0 overwrites C (NaN not propagated),
 * alpha==0 or k==0 only scales C.  (driver/level3/level3.c:229-259,
 * kernel/generic/gemm_beta.c:41-94) */
void orc_dgemm(char transa, char transb, int m, int n, int k, double alpha,
               const double *A, int lda, const double *B, int ldb, double beta,
               double *C, int ldc);
void orc_sgemm(char transa, char transb, int m, int n, int k, float alpha,
               const float *A, int lda, const float *B, int ldb, float beta,
               float *C, int ldc);

/* Same contract as orc_dgemm, but the products are summed in double-double
 * arithmetic (TwoProd by fma + TwoSum) and rounded once: a reference that is
 * accurate to ~2^-100 relative to |alpha||A||B| + |beta||C|.  Used to measure
 * the error of the native and emulated FP64 paths. */
void orc_dgemm_dd(char transa, char transb, int m, int n, int k, double alpha,
                  const double *A, int lda, const double *B, int ldb,
                  double beta, double *C, int ldc);
/* |alpha|*|op(A)|*|op(B)| + |beta|*|C|, the DMMCH "G" matrix (ctest/c_dblat3c.c:2956). */
void orc_dgemm_absbound(char transa, char transb, int m, int n, int k,
                        double alpha, const double *A, int lda, const double *B,
                        int ldb, double beta, const double *C, int ldc,
                        double *G, int ldg);

/* B <- alpha * op(A)^-1 * B (side 'L') or alpha * B * op(A)^-1 (side 'R').
 * alpha applied first; alpha==0 zeroes B. (driver/level3/trsm_L.c:103-113) */
void orc_dtrsm(char side, char uplo, char transa, char diag, int m, int n,
               double alpha, const double *A, int lda, double *B, int ldb);
void orc_strsm(char side, char uplo, char transa, char diag, int m, int n,
               float alpha, const float *A, int lda, float *B, int ldb);

/* C <- alpha*A*A^T + beta*C (trans 'N') or alpha*A^T*A + beta*C, one triangle.
 * (driver/level3/syrk_k.c:52-105) */
void orc_dsyrk(char uplo, char trans, int n, int k, double alpha,
               const double *A, int lda, double beta, double *C, int ldc);

/* Row interchanges rows k1..k2 (1-based) by ipiv with increment incx.
 * (interface/lapack/laswp.c:55-110, lapack/laswp/generic/laswp_k_1.c) */
void orc_dlaswp(int n, double *A, int lda, int k1, int k2, const int *ipiv,
                int incx);
void orc_slaswp(int n, float *A, int lda, int k1, int k2, const int *ipiv,
                int incx);

/* LU with partial pivoting; returns info (first exactly-zero pivot, 1-based).
 * Pivot = first index of max |.| (IAMAX); reciprocal scaling only when
 * |pivot| >= DBL_MIN.  (lapack/getf2/getf2_k.c:46-125,
 * lapack/getrf/getrf_single.c:47-180) */
int orc_dgetrf(int m, int n, double *A, int lda, int *ipiv);
int orc_sgetrf(int m, int n, float *A, int lda, int *ipiv);
/* (lapack/getrs/getrs_single.c:42-68) */
int orc_dgetrs(char trans, int n, int nrhs, const double *A, int lda,
               const int *ipiv, double *B, int ldb);
int orc_sgetrs(char trans, int n, int nrhs, const float *A, int lda,
               const int *ipiv, float *B, int ldb);
/* (interface/lapack/gesv.c:63-161) */
int orc_dgesv(int n, int nrhs, double *A, int lda, int *ipiv, double *B,
              int ldb);
/* Cholesky; returns info = first non-positive pivot (1-based) with that
 * pivot value written back.  (lapack/potrf/potrf_L_single.c:81-236,
 * lapack/potf2/potf2_L.c:50-97, potf2_U.c:50-94) */
int orc_dpotrf(char uplo, int n, double *A, int lda);
int orc_spotrf(char uplo, int n, float *A, int lda);

/* Mixed precision solve: FP32 LU + FP64 iterative refinement, FP64 fallback.
 * Returns info; *iter as in LAPACK (>=0 refinement steps, -2 overflow in
 * FP32 conversion, -3 FP32 LU singular, -31 no convergence in 30 steps).
 * (lapack-netlib/SRC/dsgesv.f:193-430) */
int orc_dsgesv(int n, int nrhs, double *A, int lda, int *ipiv, const double *B,
               int ldb, double *X, int ldx, int *iter);

/* ||A||_inf (max row sum). (lapack-netlib/SRC/dlange.f, NORM='I') */
double orc_dlange_inf(int m, int n, const double *A, int lda);

/* Complex GEMM on interleaved (re, im) arrays, alpha/beta -> (re, im), op
 * codes N, T, R, C.  4M semantics (interface/gemm.c with COMPLEX,
 * driver/level3/level3.c) and the 3M driver (driver/level3/gemm3m_level3.c). */
void orc_zgemm(char transa, char transb, int m, int n, int k, const double *alpha,
               const double *A, int lda, const double *B, int ldb, const double *beta,
               double *C, int ldc);
void orc_cgemm(char transa, char transb, int m, int n, int k, const float *alpha,
               const float *A, int lda, const float *B, int ldb, const float *beta, float *C,
               int ldc);
void orc_zgemm3m(char transa, char transb, int m, int n, int k, const double *alpha,
                 const double *A, int lda, const double *B, int ldb, const double *beta,
                 double *C, int ldc);
void orc_cgemm3m(char transa, char transb, int m, int n, int k, const float *alpha,
                 const float *A, int lda, const float *B, int ldb, const float *beta, float *C,
                 int ldc);

/* Grouped batch on the host cores: the per-problem oracle routines with
 * OpenMP over the problems (each problem on one thread), the CPU
 * counterpart of the grouped GPU batch.  The layout matches the library's
 * gb_batch_problem; type 0 DGEMM (C = alpha op(A) op(B) + beta C), 1 DGESV
 * (A n x n factored, B n x k solved, C = int ipiv[n], *info), 2 DPOTRF
 * (uplo 'L'/'U', *info).  driver/level3/gemm_batch_thread.c:79-156 threads
 * cblas_dgemm_batch over problems the same way. */
typedef struct orc_batch_problem {
  int type;
  int m, n, k;
  char transa, transb, uplo, pad;
  double alpha, beta;
  void *A, *B, *C;
  int lda, ldb, ldc;
  int *info;
} orc_batch_problem;
void orc_batch(const orc_batch_problem *probs, int count);

#ifdef __cplusplus
}
#endif
#endif
