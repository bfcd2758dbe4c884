/*
 * gbblas.h -- C ABI of libgbblas, a GB300 (sm_103a) implementation of
 * OpenBLAS's level-3 BLAS and blocked-LAPACK hot path.
 *
 * Part 1 declares the drop-in entry points with exactly the prototypes of
 * OpenBLAS's cblas.h and Fortran-77 interface (column-major, transpose and
 * leading-dimension semantics, xerbla error reporting, LAPACK `info`).  Each
 * declaration names the reference interface it replaces (paths relative to
 * the OpenBLAS source tree).  These entry points take HOST pointers, copy
 * operands to the GPU, compute there and copy results back before returning
 * (blocking BLAS semantics).  Pointers that are already device memory are
 * detected and used in place.
 *
 * Part 2 declares device-pointer variants (gb_*_dev) that only enqueue work
 * on the library stream, plus control functions (stream, precision mode,
 * error state).  No entry point takes framework-specific types: plain
 * pointers, 32/64-bit integers and an opaque stream handle.
 */
#ifndef GBBLAS_H
#define GBBLAS_H

#include <stdint.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif
#ifdef __cplusplus
extern "C" {
#endif

typedef int blasint; /* common.h:270-277 (32-bit unless INTERFACE64) */

/* cblas.h:62-66 */
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113,
                       CblasConjNoTrans = 114 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };
typedef enum CBLAS_ORDER CBLAS_ORDER;
typedef enum CBLAS_TRANSPOSE CBLAS_TRANSPOSE;
typedef enum CBLAS_UPLO CBLAS_UPLO;
typedef enum CBLAS_DIAG CBLAS_DIAG;
typedef enum CBLAS_SIDE CBLAS_SIDE;

/* ======================================================================= */
/* Part 1: drop-in entry points (host pointers, blocking)                   */
/* ======================================================================= */

/* replaces cblas_dgemm, interface/gemm.c:294-651 (cblas.h:300-301) */
void cblas_dgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA,
                 enum CBLAS_TRANSPOSE TransB, blasint M, blasint N, blasint K,
                 double alpha, const double *A, blasint lda, const double *B,
                 blasint ldb, double beta, double *C, blasint ldc);
/* replaces cblas_sgemm, interface/gemm.c (FP32 build; cblas.h:298-299) */
void cblas_sgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA,
                 enum CBLAS_TRANSPOSE TransB, blasint M, blasint N, blasint K,
                 float alpha, const float *A, blasint lda, const float *B,
                 blasint ldb, float beta, float *C, blasint ldc);
/* replaces cblas_dtrsm, interface/trsm.c:213-412 (cblas.h:358-359) */
void cblas_dtrsm(enum CBLAS_ORDER Order, enum CBLAS_SIDE Side,
                 enum CBLAS_UPLO Uplo, enum CBLAS_TRANSPOSE TransA,
                 enum CBLAS_DIAG Diag, blasint M, blasint N, double alpha,
                 const double *A, blasint lda, double *B, blasint ldb);
/* replaces cblas_dsyrk, interface/syrk.c:195-402 (cblas.h:331-332) */
void cblas_dsyrk(enum CBLAS_ORDER Order, enum CBLAS_UPLO Uplo,
                 enum CBLAS_TRANSPOSE Trans, blasint N, blasint K, double alpha,
                 const double *A, blasint lda, double beta, double *C,
                 blasint ldc);
/* replaces cblas_dtrmm, interface/trsm.c built as TRMM (cblas.h:349-350) */
void cblas_dtrmm(enum CBLAS_ORDER Order, enum CBLAS_SIDE Side, enum CBLAS_UPLO Uplo,
                 enum CBLAS_TRANSPOSE TransA, enum CBLAS_DIAG Diag, blasint M, blasint N,
                 double alpha, const double *A, blasint lda, double *B, blasint ldb);
/* replaces cblas_dsyr2k, interface/syr2k.c (cblas.h:340-341) */
void cblas_dsyr2k(enum CBLAS_ORDER Order, enum CBLAS_UPLO Uplo, enum CBLAS_TRANSPOSE Trans,
                  blasint N, blasint K, double alpha, const double *A, blasint lda,
                  const double *B, blasint ldb, double beta, double *C, blasint ldc);
/* replaces cblas_dgemmt, interface/gemmt.c (cblas.h:313-314) */
void cblas_dgemmt(enum CBLAS_ORDER Order, enum CBLAS_UPLO Uplo, enum CBLAS_TRANSPOSE TransA,
                  enum CBLAS_TRANSPOSE TransB, blasint M, blasint K, double alpha,
                  const double *A, blasint lda, const double *B, blasint ldb, double beta,
                  double *C, blasint ldc);
/* replace cblas_zgemm / cblas_cgemm / cblas_zgemm3m / cblas_cgemm3m,
 * interface/gemm.c compiled with COMPLEX (and GEMM3M), cblas.h:302-309:
 * alpha and beta point to (re, im); TransA/TransB may be CblasConjNoTrans and
 * CblasConjTrans; arrays hold interleaved complex elements. */
void cblas_zgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA,
                 enum CBLAS_TRANSPOSE TransB, blasint M, blasint N, blasint K,
                 const void *alpha, const void *A, blasint lda, const void *B,
                 blasint ldb, const void *beta, void *C, blasint ldc);
void cblas_cgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA,
                 enum CBLAS_TRANSPOSE TransB, blasint M, blasint N, blasint K,
                 const void *alpha, const void *A, blasint lda, const void *B,
                 blasint ldb, const void *beta, void *C, blasint ldc);
void cblas_zgemm3m(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA,
                   enum CBLAS_TRANSPOSE TransB, blasint M, blasint N, blasint K,
                   const void *alpha, const void *A, blasint lda, const void *B,
                   blasint ldb, const void *beta, void *C, blasint ldc);
void cblas_cgemm3m(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA,
                   enum CBLAS_TRANSPOSE TransB, blasint M, blasint N, blasint K,
                   const void *alpha, const void *A, blasint lda, const void *B,
                   blasint ldb, const void *beta, void *C, blasint ldc);
/* replaces cblas_dgemm_batch, interface/gemm_batch.c:117-372 (cblas.h:422-423) */
void cblas_dgemm_batch(enum CBLAS_ORDER Order,
                       const enum CBLAS_TRANSPOSE *TransA_array,
                       const enum CBLAS_TRANSPOSE *TransB_array,
                       const blasint *M_array, const blasint *N_array,
                       const blasint *K_array, const double *alpha_array,
                       const double **A_array, const blasint *lda_array,
                       const double **B_array, const blasint *ldb_array,
                       const double *beta_array, double **C_array,
                       const blasint *ldc_array, blasint group_count,
                       const blasint *group_size);

/* replaces dgemm_, interface/gemm.c:181-290 (common_interface.h) */
void dgemm_(const char *TRANSA, const char *TRANSB, const blasint *M,
            const blasint *N, const blasint *K, const double *alpha,
            const double *A, const blasint *ldA, const double *B,
            const blasint *ldB, const double *beta, double *C,
            const blasint *ldC);
/* replaces sgemm_, interface/gemm.c:181-290 (FP32 build) */
void sgemm_(const char *TRANSA, const char *TRANSB, const blasint *M,
            const blasint *N, const blasint *K, const float *alpha,
            const float *A, const blasint *ldA, const float *B,
            const blasint *ldB, const float *beta, float *C,
            const blasint *ldC);
/* replace zgemm_ / cgemm_ (interface/gemm.c:181-290 compiled with COMPLEX,
 * common_interface.h:492-495) and zgemm3m_ / cgemm3m_ (the same file with
 * GEMM3M, common_interface.h:499-502): TRANSA/TRANSB in N, T, R (conjugate,
 * no transpose), C (conjugate transpose); alpha/beta point to (re, im). */
void zgemm_(const char *TRANSA, const char *TRANSB, const blasint *M,
            const blasint *N, const blasint *K, const double *alpha,
            const double *A, const blasint *ldA, const double *B,
            const blasint *ldB, const double *beta, double *C,
            const blasint *ldC);
void cgemm_(const char *TRANSA, const char *TRANSB, const blasint *M,
            const blasint *N, const blasint *K, const float *alpha,
            const float *A, const blasint *ldA, const float *B,
            const blasint *ldB, const float *beta, float *C,
            const blasint *ldC);
void zgemm3m_(const char *TRANSA, const char *TRANSB, const blasint *M,
              const blasint *N, const blasint *K, const double *alpha,
              const double *A, const blasint *ldA, const double *B,
              const blasint *ldB, const double *beta, double *C,
              const blasint *ldC);
void cgemm3m_(const char *TRANSA, const char *TRANSB, const blasint *M,
              const blasint *N, const blasint *K, const float *alpha,
              const float *A, const blasint *ldA, const float *B,
              const blasint *ldB, const float *beta, float *C,
              const blasint *ldC);
/* replaces dtrsm_, interface/trsm.c:114-209 */
void dtrsm_(const char *SIDE, const char *UPLO, const char *TRANSA,
            const char *DIAG, const blasint *M, const blasint *N,
            const double *alpha, const double *A, const blasint *ldA,
            double *B, const blasint *ldB);
/* replaces dtrmm_, interface/trsm.c built as TRMM (B = alpha*op(A)*B or
 * alpha*B*op(A), A triangular) */
void dtrmm_(const char *SIDE, const char *UPLO, const char *TRANSA, const char *DIAG,
            const blasint *M, const blasint *N, const double *alpha, const double *A,
            const blasint *ldA, double *B, const blasint *ldB);
/* replaces dsyr2k_, interface/syr2k.c:96-191 (C = alpha*A*B' + alpha*B*A' + beta*C
 * on one triangle) */
void dsyr2k_(const char *UPLO, const char *TRANS, const blasint *N, const blasint *K,
             const double *alpha, const double *A, const blasint *ldA, const double *B,
             const blasint *ldB, const double *beta, double *C, const blasint *ldC);
/* replaces dgemmt_, interface/gemmt.c:80-200 (C = alpha*op(A)*op(B) + beta*C on
 * one triangle of the M x M matrix C) */
void dgemmt_(const char *UPLO, const char *TRANSA, const char *TRANSB, const blasint *M,
             const blasint *K, const double *alpha, const double *A, const blasint *ldA,
             const double *B, const blasint *ldB, const double *beta, double *C,
             const blasint *ldC);
/* replaces dsyrk_, interface/syrk.c:96-191 */
void dsyrk_(const char *UPLO, const char *TRANS, const blasint *N,
            const blasint *K, const double *alpha, const double *A,
            const blasint *ldA, const double *beta, double *C,
            const blasint *ldC);

/* replaces dgetrf_, interface/lapack/getrf.c:53-133 */
int dgetrf_(const blasint *M, const blasint *N, double *A, const blasint *ldA,
            blasint *ipiv, blasint *Info);
/* replaces dgetrs_, interface/lapack/getrs.c:63-152 */
int dgetrs_(const char *TRANS, const blasint *N, const blasint *NRHS,
            const double *A, const blasint *ldA, const blasint *ipiv,
            double *B, const blasint *ldB, blasint *Info);
/* replaces dgesv_, interface/lapack/gesv.c:63-161 */
int dgesv_(const blasint *N, const blasint *NRHS, double *A, const blasint *ldA,
           blasint *ipiv, double *B, const blasint *ldB, blasint *Info);
/* replaces dpotrf_, interface/lapack/potrf.c:63-150 */
int dpotrf_(const char *UPLO, const blasint *N, double *A, const blasint *ldA,
            blasint *Info);
/* replaces dlaswp_, interface/lapack/laswp.c:55-110 */
int dlaswp_(const blasint *N, double *A, const blasint *LDA, const blasint *K1,
            const blasint *K2, const blasint *ipiv, const blasint *INCX);
/* replaces dsgesv_ (netlib, compiled into OpenBLAS),
 * lapack-netlib/SRC/dsgesv.f:193-430.  SWORK/WORK are accepted for ABI
 * compatibility; the GPU path keeps its own workspace. */
int dsgesv_(const blasint *N, const blasint *NRHS, double *A, const blasint *ldA,
            blasint *ipiv, const double *B, const blasint *ldB, double *X,
            const blasint *ldX, double *WORK, float *SWORK, blasint *ITER,
            blasint *Info);
/* replaces dpotrs_ (netlib, compiled into OpenBLAS),
 * lapack-netlib/SRC/dpotrs.f:109-160: A X = B with the Cholesky factor of
 * dpotrf_. */
int dpotrs_(const char *UPLO, const blasint *N, const blasint *NRHS, const double *A,
            const blasint *ldA, double *B, const blasint *ldB, blasint *Info);
/* replaces dsposv_ (netlib, compiled into OpenBLAS),
 * lapack-netlib/SRC/dsposv.f:199-434: FP32 Cholesky + FP64 refinement with
 * the FP64 DPOTRF/DPOTRS fallback and dsposv's ITER codes.  WORK/SWORK are
 * accepted for ABI compatibility; the GPU path keeps its own workspace. */
int dsposv_(const char *UPLO, const blasint *N, const blasint *NRHS, double *A,
            const blasint *ldA, const double *B, const blasint *ldB, double *X,
            const blasint *ldX, double *WORK, float *SWORK, blasint *ITER,
            blasint *Info);

/* replaces xerbla_, driver/others/xerbla.c:56-64.  Weak: an application may
 * define its own.  Prints " ** On entry to %6s parameter number %2d had an
 * illegal value" and returns. */
int xerbla_(const char *name, const blasint *info, blasint len);

/* ======================================================================= */
/* Part 2: GB300-native API (device pointers, stream-ordered)               */
/* ======================================================================= */

/* status codes returned by gb_* functions */
#define GB_SUCCESS 0
#define GB_ERR_INVALID_VALUE 1 /* argument error (xerbla also called) */
#define GB_ERR_CUDA 2          /* a CUDA runtime/driver call failed */
#define GB_ERR_NO_DEVICE 3     /* no usable CUDA device */
#define GB_ERR_ALLOC 4         /* device or pinned allocation failed */
#define GB_ERR_KERNEL 5        /* a kernel reported an error (e.g. bounded wait expired) */
#define GB_ERR_UNSUPPORTED 6   /* shape/option outside what the kernels support */

/* DGEMM precision modes */
#define GB_DGEMM_NATIVE 0   /* FP64 FMA units */
#define GB_DGEMM_EMULATED 1 /* Ozaki schemes (residues or 8-bit slices) on bf16 tensor cores */
#define GB_DGEMM_AUTO 2     /* emulated from m*n*k >= 384^3 (k >= 64), native below */

/* Stream used by every entry point of the calling thread (NULL = the
 * library's own non-blocking stream).  The handle is a cudaStream_t. */
int gb_set_stream(void *stream);
void *gb_get_stream(void);
/* Block until all work queued by this thread's entry points is done and
 * report any kernel-side error. */
int gb_synchronize(void);
/* Status and message of the calling thread's last error (message may be NULL). */
int gb_last_error(char *msg, int len);
void gb_clear_error(void);
/* Last argument error seen by xerbla on this thread: routine name (up to 8
 * chars + NUL) and parameter position; returns that position or 0. */
int gb_last_xerbla(char *name, int len);
/* Precision of the FP64 GEMM behind cblas_dgemm/dgemm_, the GEMMs inside
 * dsyrk_/dtrmm_/dsyr2k_/dgemmt_/zgemm_, the LU and Cholesky trailing updates,
 * and the form of dtrsm_ (emulated: recursive, 128-wide triangles solved in
 * FP64, the rest on the emulated GEMM); default from GB_DGEMM_MODE. */
int gb_set_dgemm_mode(int mode);
int gb_get_dgemm_mode(void);
/* FP32 GEMM behind sgemm_/cblas_sgemm and the FP32 LU of the mixed solver
 * (default from GB_SGEMM_MODE=auto|simt|tensor).  The tensor form splits
 * each operand into three bf16 terms and runs six products on the tensor
 * cores with FP32 accumulation (FP32-level accuracy). */
#define GB_SGEMM_AUTO 0   /* tensor cores when the shape fills the GPU */
#define GB_SGEMM_SIMT 1   /* FP32 FMA units */
#define GB_SGEMM_TENSOR 2 /* always the bf16x3 tensor-core form */
int gb_set_sgemm_mode(int mode);
int gb_get_sgemm_mode(void);
/* Slice count of the emulated DGEMM behind dgemm_/cblas_dgemm and the other
 * caller-facing GEMMs (1..8 fixed).  0 (the default; GB_OZAKI_SLICES=auto)
 * chooses per 256-column tile of C on the device, from worst-case bounds on
 * every column's error measured against GB_OZAKI_TOL (default 8) x 2^-52
 * times that column's sum_i (|A||B|)_ij:
 *  - the modular scheme (unless turned off, below) when its bound
 *      sum_i |dC_ij| <= 2^-t (T_e ||b_j||_1 + 2^f_j (T_1 + 2^-t k T_e)) + roundings
 *    meets the tolerance: op(A) and op(B) cut to t-bit integers (t = 56 for a
 *    K segment of 4096), their product computed exactly from 14 residue
 *    products (moduli 461..511, residues on the bf16 tensor cores) and the
 *    Chinese remainder theorem;
 *  - otherwise the smallest slice count S of the digit-slice scheme with
 *      sum_i |dC_ij| <= 2^-8S (T_e ||b_j||_1 + 2^f_j (T_1 + 7.06 k T_e)) + roundings
 *    within the tolerance (S(S+1)/2 slice products; 8 is the most there is).
 * (2^f_j: column j's scale, T_e: the sum of the rows' scales, T_1 = sum |A|,
 * k: the K segment.)  Uniform and exponent-spread operands take the
 * modular scheme; digit slices (8) are left for columns whose error bound it
 * cannot meet, e.g. rows scaled far above the entries that meet the column.
 * The LU/Cholesky trailing updates, panel solves and refinement residuals
 * use the modular scheme on every tile when their depth k is 512 or more,
 * and 7 digit slices otherwise (or when the calling thread has turned the
 * modular scheme off). */
int gb_set_ozaki_slices(int slices);
/* Largest slice count chosen by the calling thread's last automatic-mode
 * emulated DGEMM for its digit-slice tiles (0 if none); synchronises the
 * thread's stream. */
int gb_last_ozaki_slices(void);
/* Moduli used by the calling thread's last automatic-mode emulated DGEMM
 * (14 when any tile took the modular scheme, else 0); synchronises the
 * thread's stream. */
int gb_last_ozaki_moduli(void);
/* Automatic mode's modular scheme for the calling thread: 1 allowed (the
 * default; GB_OZAKI_MODULAR=0 changes it), 0 digit slices only. */
int gb_set_ozaki_modular(int on);
/* Library version string. */
const char *gb_version(void);

/* Instrumentation.  gb_kernel_launches: number of CUDA kernels this library
 * has launched (all threads) since it was loaded.  gb_profile_enable(1)
 * brackets the dominant kernel of each call (e.g. "slice_gemm") with CUDA
 * events on the launching stream; gb_profile_kernel_ms synchronises, returns
 * the summed duration of the named kernel and its launch count, and resets
 * the record when `reset` is non-zero. */
int64_t gb_kernel_launches(void);
int gb_profile_enable(int on);
double gb_profile_kernel_ms(const char *name, int *launches, int reset);

/* C <- alpha*op(A)*op(B) + beta*C, all device pointers, column-major,
 * trans 'N'/'T'/'C'.  Uses the current DGEMM mode. */
int gb_dgemm_dev(char transa, char transb, int64_t m, int64_t n, int64_t k,
                 double alpha, const double *A, int64_t lda, const double *B,
                 int64_t ldb, double beta, double *C, int64_t ldc);
/* Native FP64 GEMM regardless of mode. */
int gb_dgemm_native_dev(char transa, char transb, int64_t m, int64_t n,
                        int64_t k, double alpha, const double *A, int64_t lda,
                        const double *B, int64_t ldb, double beta, double *C,
                        int64_t ldc);
/* Emulated FP64 GEMM with `slices` 8-bit slices per operand (1..8; 0 = the
 * thread's setting, automatic unless fixed by gb_set_ozaki_slices). */
int gb_dgemm_emulated_dev(char transa, char transb, int64_t m, int64_t n,
                          int64_t k, double alpha, const double *A, int64_t lda,
                          const double *B, int64_t ldb, double beta, double *C,
                          int64_t ldc, int slices);
int gb_sgemm_dev(char transa, char transb, int64_t m, int64_t n, int64_t k,
                 float alpha, const float *A, int64_t lda, const float *B,
                 int64_t ldb, float beta, float *C, int64_t ldc);
int gb_dtrsm_dev(char side, char uplo, char transa, char diag, int64_t m,
                 int64_t n, double alpha, const double *A, int64_t lda,
                 double *B, int64_t ldb);
int gb_dtrmm_dev(char side, char uplo, char transa, char diag, int64_t m, int64_t n,
                 double alpha, const double *A, int64_t lda, double *B, int64_t ldb);
int gb_dsyr2k_dev(char uplo, char trans, int64_t n, int64_t k, double alpha, const double *A,
                  int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                  int64_t ldc);
int gb_dgemmt_dev(char uplo, char transa, char transb, int64_t m, int64_t k, double alpha,
                  const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                  double *C, int64_t ldc);
/* Complex GEMM on device pointers (interleaved complex arrays); alpha/beta
 * are HOST pointers to (re, im).  zgemm: one real GEMM on the [Ar -Ai; Ai Ar]
 * embedding with the current DGEMM mode; 3m: three real products. */
int gb_zgemm_dev(char transa, char transb, int64_t m, int64_t n, int64_t k,
                 const double *alpha, const double *A, int64_t lda,
                 const double *B, int64_t ldb, const double *beta, double *C,
                 int64_t ldc);
int gb_cgemm_dev(char transa, char transb, int64_t m, int64_t n, int64_t k,
                 const float *alpha, const float *A, int64_t lda,
                 const float *B, int64_t ldb, const float *beta, float *C,
                 int64_t ldc);
int gb_zgemm3m_dev(char transa, char transb, int64_t m, int64_t n, int64_t k,
                   const double *alpha, const double *A, int64_t lda,
                   const double *B, int64_t ldb, const double *beta, double *C,
                   int64_t ldc);
int gb_cgemm3m_dev(char transa, char transb, int64_t m, int64_t n, int64_t k,
                   const float *alpha, const float *A, int64_t lda,
                   const float *B, int64_t ldb, const float *beta, float *C,
                   int64_t ldc);
int gb_dsyrk_dev(char uplo, char trans, int64_t n, int64_t k, double alpha,
                 const double *A, int64_t lda, double beta, double *C,
                 int64_t ldc);
/* LU with partial pivoting; ipiv (int32, 1-based, min(m,n) entries) and
 * info (one int32) are device pointers written by the GPU. */
int gb_dgetrf_dev(int64_t m, int64_t n, double *A, int64_t lda, int *ipiv,
                  int *info);
int gb_dgetrs_dev(char trans, int64_t n, int64_t nrhs, const double *A,
                  int64_t lda, const int *ipiv, double *B, int64_t ldb);
/* FP32 LU and solve (the factorisation behind the mixed solver; sgetrf_ /
 * sgetrs_ semantics, interface/lapack/getrf.c, getrs.c, single precision). */
int gb_sgetrf_dev(int64_t m, int64_t n, float *A, int64_t lda, int *ipiv,
                  int *info);
int gb_sgetrs_dev(char trans, int64_t n, int64_t nrhs, const float *A,
                  int64_t lda, const int *ipiv, float *B, int64_t ldb);
/* Row interchanges k1..k2 (1-based) of an n-column device matrix using a
 * device ipiv vector with increment incx (+1 or -1 for the fast path). */
int gb_dlaswp_dev(int64_t n, double *A, int64_t lda, int64_t k1, int64_t k2,
                  const int *ipiv, int64_t incx);
int gb_dpotrf_dev(char uplo, int64_t n, double *A, int64_t lda, int *info);
/* Solve with a Cholesky factor from gb_dpotrf_dev (device pointers). */
int gb_dpotrs_dev(char uplo, int64_t n, int64_t nrhs, const double *A, int64_t lda,
                  double *B, int64_t ldb);
/* Grouped batches of small, uneven problems in one persistent launch (the
 * reference's cblas_dgemm_batch, interface/gemm_batch.c, extended to LU solves
 * and Cholesky).  All pointers are device pointers.  type selects:
 *   GB_BATCH_DGEMM : C = alpha*op(A)*op(B) + beta*C (m, n, k, transa/transb)
 *   GB_BATCH_DGESV : A (n x n) overwritten by its LU, B (n x k right-hand
 *                    sides) by the solution, C = int ipiv[n], *info
 *   GB_BATCH_DPOTRF: Cholesky of A (n x n, uplo 'L'/'U'), *info
 * A plan uploads the table, orders it by cost and captures the launch in a
 * CUDA graph; gb_batch_execute replays it on the thread's stream.
 * GB_BATCH_MIXED solves the DGESV problems with an FP32 LU and FP64
 * refinement (FP64 fallback per problem).  gb_batch_plan_tune times the
 * candidate CTA sizes on the batch itself (it executes the batch, so inputs
 * must be re-initialised afterwards) and caches the winner for batches with
 * the same size histogram.  gb_batch_execute_loop runs the same per-problem
 * code with one launch per problem (the comparison baseline).  The tuner also
 * picks the DGEMM tile (32x32 or 64x64) per size bin; DGESV and DPOTRF orders
 * are limited to 12288. */
#define GB_BATCH_DGEMM 0
#define GB_BATCH_DGESV 1
#define GB_BATCH_DPOTRF 2
#define GB_BATCH_MIXED 1
/* flag: the DGEMM problems run on the emulated-FP64 kernel (Ozaki split into
 * seven 8-bit digit slices multiplied on the bf16 tensor cores, FP64-level
 * accuracy; K up to 4096 and m, n up to 2048: larger problems and tiles
 * holding Inf/NaN use the FP64 loop) */
#define GB_BATCH_EMULATED 2
typedef struct gb_batch_problem {
  int type;
  int m, n, k;
  char transa, transb, uplo, pad;
  double alpha, beta;
  void *A, *B, *C;
  int lda, ldb, ldc;
  int *info;
} gb_batch_problem;
void *gb_batch_plan_create(const gb_batch_problem *problems, int count, int flags);
int gb_batch_plan_tune(void *plan);
int gb_batch_plan_threads(void *plan);
int gb_batch_execute(void *plan);
int gb_batch_execute_loop(void *plan);
void gb_batch_plan_destroy(void *plan);

/* LU with partial pivoting that allocates no device memory.  This entry has
 * no counterpart in the reference.  It exists for callers that cannot let a
 * library allocate: applications that hand all of HBM to their own arena and
 * forbid other allocations, services held to a fixed memory budget, and loops
 * that cannot absorb the synchronisation and latency of cudaMalloc/cudaFree.
 * Same contract as gb_dgetrf_dev (native FP64 trailing updates), on the given
 * stream (NULL = the legacy default stream).  Its scratch is a 1 MiB
 * file-scope device array inside the library, held by every GPU that loads
 * the library until the process exits.  The array has candidate slots for
 * 1024 blocks of the grid-wide panel kernel, so m is limited to the rows one
 * panel can cover on the device: 524288 at most, fewer where fewer of those
 * blocks can be co-resident (the cluster panel covers up to 8192 rows without
 * slots).  A larger m is rejected with GB_ERR_UNSUPPORTED before any work is
 * queued; the error message states the device's limit.  The first call on
 * each device looks up the array's device address with that device current;
 * make that first call before any stream capture.  All calls share the array:
 * calls whose GPU work overlaps (other streams, other threads) race and must
 * be serialised by the caller.  The panel kernel's bounded grid barrier keeps
 * its status word in that array too; if one of its waits ever gives up, the
 * call sets *info to GB_INFO_WAIT_EXPIRED (a negative value no argument check
 * produces) and the factors are incomplete. */
#define GB_INFO_WAIT_EXPIRED (-1000)
int gb_dgetrf_noalloc_dev(int64_t m, int64_t n, double *A, int64_t lda,
                          int *ipiv, int *info, void *stream);
/* Mixed-precision solve (FP32 LU on the GPU + FP64 refinement, GMRES-IR
 * when plain refinement stalls, FP64 LU fallback).  Device pointers except
 * iter/info, which are host outputs (this call synchronises).  A is only
 * overwritten (with its FP64 LU) when the solve falls back to FP64, as in
 * dsgesv.  iter follows dsgesv (>= 0 refinement steps, < 0 fallback reason);
 * a solve finished by GMRES-IR reports 100 + GMRES iterations. */
int gb_dsgesv_dev(int64_t n, int64_t nrhs, double *A, int64_t lda, int *ipiv,
                  const double *B, int64_t ldb, double *X, int64_t ldx,
                  int *iter, int *info);
/* Mixed-precision Cholesky solve of a symmetric positive definite A (stored
 * triangle `uplo`): FP32 Cholesky on the GPU + FP64 refinement, FP64
 * Cholesky fallback (dsposv semantics and ITER codes).  Device pointers
 * except iter/info (host outputs; this call synchronises).  A is only
 * overwritten (with its FP64 factor) on a fallback. */
int gb_dsposv_dev(char uplo, int64_t n, int64_t nrhs, double *A, int64_t lda,
                  const double *B, int64_t ldb, double *X, int64_t ldx, int *iter,
                  int *info);

#ifdef __cplusplus
}
#endif
#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#endif /* GBBLAS_H */
