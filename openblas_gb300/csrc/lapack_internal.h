// Internal interfaces of the LAPACK drivers (LU, Cholesky, solves).
#pragma once

#include "gb_internal.h"

namespace gb {

// Width of a panel factored by the cooperative panel kernel; also the
// diagonal-block size of the triangular solves that follow it.
constexpr int PANEL_NB = 32;

// Kernel error codes written to the context status word.
constexpr int GB_KERR_BARRIER_TIMEOUT = 1;
constexpr int GB_KERR_MBARRIER_TIMEOUT = 2;
constexpr int GB_KERR_CLUSTER_TIMEOUT = 4;  // a cluster panel CTA waited too long for a message
constexpr int GB_KERR_CHAIN_TIMEOUT = 3;  // a solve block waited too long for its predecessor

// LU with partial pivoting of an m x n matrix (device pointers).  ipiv gets
// min(m,n) 1-based global row indices, *info the first zero pivot (1-based)
// or 0.  Semantics of lapack/getrf/getrf_single.c + getf2_k.c.
template <typename T>
int getrf_device(int64_t m, int64_t n, T *A, int64_t lda, int *ipiv, int *info, cudaStream_t s);
// gemm_mode 1 (double only): the trailing updates run on the emulated-FP64
// GEMM (FP64-accurate, tensor cores); 0: native FP64 / FP32 SIMT GEMM.
template <typename T>
int getrf_device_mode(int64_t m, int64_t n, T *A, int64_t lda, int *ipiv, int *info,
                      int gemm_mode, cudaStream_t s);
// Solve op(A) X = B with an LU from getrf_device (lapack/getrs/getrs_single.c).
template <typename T>
int getrs_device(int trans, int64_t n, int64_t nrhs, const T *A, int64_t lda, const int *ipiv,
                 T *B, int64_t ldb, cudaStream_t s);
// Row interchanges k1..k2 (1-based) over n columns (lapack/laswp/generic).
template <typename T>
int laswp_device(int64_t n, T *A, int64_t lda, int64_t k1, int64_t k2, const int *ipiv,
                 int64_t incx, cudaStream_t s);
// Inverses of the 64x64 diagonal blocks of the unit-lower L and of U of an
// LU factorisation (each n/64 * 64*64 entries), and the solve that uses them
// (interchanges applied beforehand): one launch per triangle, 64-row blocks
// chained through release/acquire flags.
template <typename T>
int lu_block_inverses(int64_t n, const T *A, int64_t lda, T *Linv, T *Uinv, cudaStream_t s);
template <typename T>
int lu_block_solve(int64_t n, int64_t nrhs, const T *A, int64_t lda, const T *Linv,
                   const T *Uinv, T *B, int64_t ldb, cudaStream_t s);
// Cholesky forms: inverses of the non-unit diagonal blocks of both triangles,
// and the mirror of one strict triangle onto the other (transposed), after
// which lu_block_solve applies L then L^T (or U^T then U).
template <typename T>
int chol_block_inverses(int64_t n, const T *A, int64_t lda, T *Linv, T *Uinv, cudaStream_t s);
template <typename T>
int mirror_triangle(int64_t n, T *A, int64_t lda, int from_lower, cudaStream_t s);
// Solve A X = B with a Cholesky factor from potrf_device (lapack/potrs:
// two triangular solves).
int potrs_device(int uplo, int64_t n, int64_t nrhs, const double *A, int64_t lda, double *B,
                 int64_t ldb, cudaStream_t s);
// Final permutation of the interchanges ipiv[0..n): row i of P*B is row
// perm[i] of B; and the gather dst = P*src.
int pivots_to_perm(int64_t n, const int *ipiv, int *perm, cudaStream_t s);
template <typename T>
int apply_perm(int64_t n, int64_t ncol, const int *perm, const T *src, int64_t lds, T *dst,
               int64_t ldd, cudaStream_t s);

// Cholesky (lapack/potrf/potrf_{L,U}_single.c); *info_dev receives info.
// gemm_mode 1: trailing updates on the emulated-FP64 GEMM.
int potrf_device(int uplo, int64_t n, double *A, int64_t lda, int *info_dev, int gemm_mode,
                 cudaStream_t s);
// FP32 Cholesky (same blocking; trailing updates on the tensor-core FP32 GEMM
// when large, per the SGEMM mode).
int spotrf_device(int uplo, int64_t n, float *A, int64_t lda, int *info_dev, cudaStream_t s);

int dtrsm_device(int side, int uplo, int trans, int unit, int64_t m, int64_t n, double alpha,
                 const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s);
int strsm_device(int side, int uplo, int trans, int unit, int64_t m, int64_t n, float alpha,
                 const float *A, int64_t lda, float *B, int64_t ldb, cudaStream_t s);
int dtrsm_device_skip(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                      double alpha, const double *A, int64_t lda, double *B, int64_t ldb,
                      cudaStream_t s, const int *skip);
int dsyrk_device_skip(int uplo, int trans, int64_t n, int64_t k, double alpha, const double *A,
                      int64_t lda, double beta, double *C, int64_t ldc, cudaStream_t s,
                      const int *skip);
int strsm_device_skip(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                      float alpha, const float *A, int64_t lda, float *B, int64_t ldb,
                      cudaStream_t s, const int *skip);
int ssyrk_device_skip(int uplo, int trans, int64_t n, int64_t k, float alpha, const float *A,
                      int64_t lda, float beta, float *C, int64_t ldc, cudaStream_t s,
                      const int *skip);
int dsyrk_device(int uplo, int trans, int64_t n, int64_t k, double alpha, const double *A,
                 int64_t lda, double beta, double *C, int64_t ldc, cudaStream_t s);
// DTRSM with the engine the DGEMM mode selects (the caller-facing entries).
int dtrsm_select(int side, int uplo, int trans, int unit, int64_t m, int64_t n, double alpha,
                 const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s);

}  // namespace gb
