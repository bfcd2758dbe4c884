// Level-3 routines around the GEMM engines: DGEMMT (interface/gemmt.c),
// DSYR2K (interface/syr2k.c, driver/level3/level3_syr2k.c) and DTRMM
// (interface/trsm.c compiled as TRMM, driver/level3/trmm_L.c / trmm_R.c).
//
// All three run on the same FP64 GEMMs as DGEMM -- the native DFMA kernel,
// or, when the DGEMM mode asks for it, the emulated-FP64 (Ozaki) GEMM --
// restricted to one triangle of C where the routine stores only one:
//   DGEMMT  C_tri = alpha op(A) op(B) + beta C_tri           (one masked GEMM)
//   DSYR2K  C_tri = alpha op(A) op(B)^T + alpha op(B) op(A)^T + beta C_tri
//                                                             (two masked GEMMs)
//   DTRMM   B = alpha op(T) B  or  alpha B op(T), T the triangle of A with
//           zeros elsewhere (and ones on the diagonal for 'U'): T and a copy
//           of B are formed in scratch and one GEMM writes B.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_internal.h"
#include "lapack_internal.h"

extern "C" int gb_get_ozaki_slices_internal(void);

namespace gb {

namespace {

// T = the uplo triangle of A (uplo 0 upper, 1 lower), zeros elsewhere;
// unit_code 0 puts ones on the diagonal (the diagonal of A is not read).
__global__ void tri_copy_kernel(int64_t n, const double *__restrict__ A, int64_t lda, int uplo,
                                int unit_code, double *__restrict__ T) {
  const int64_t total = n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / n, i = e - j * n;
    double v = 0.0;
    if (i == j) v = unit_code == 0 ? 1.0 : A[i + j * lda];
    else if (uplo == 1 ? i > j : i < j) v = A[i + j * lda];
    T[e] = v;
  }
}


}  // namespace

// The FP64 GEMM the thread's DGEMM mode selects for an m x n x k product:
// emulated, native, or in auto mode the emulated one from 384^3 on (with
// k >= 64).  Measured on GB300 (device pointers, square): native 0.041 /
// 0.108 / 0.270 ms against emulated 0.096 / 0.103 / 0.108 ms at 256 / 384 /
// 512; the emulated engine's fixed cost is ~0.09 ms.
bool dgemm_mode_emulated(int64_t m, int64_t n, int64_t k) {
  const int mode = gb_get_dgemm_mode();
  return mode == GB_DGEMM_EMULATED ||
         (mode == GB_DGEMM_AUTO && (double)m * n * k >= 384.0 * 384.0 * 384.0 && k >= 64);
}

// C = alpha op(A) op(B) + beta C on a triangle of C (tri 0 full, 1 lower,
// 2 upper) with the FP64 GEMM the DGEMM mode selects; assumes k > 0 and
// alpha != 0.
int dgemm_select(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha, const double *A,
                 int64_t lda, const double *B, int64_t ldb, double beta, double *C, int64_t ldc,
                 int tri, cudaStream_t s) {
  if (dgemm_mode_emulated(m, n, k))
    return dgemm_emulated(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                          ozaki_caller_slices(), s, tri);
  launch_dgemm_fp64_tri(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, s, nullptr);
  return check_cuda(cudaGetLastError(), "gemm launch");
}

int dgemmt_device(int uplo, int ta, int tb, int64_t m, int64_t k, double alpha, const double *A,
                  int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                  int64_t ldc, cudaStream_t s) {
  if (m == 0) return GB_SUCCESS;
  const int tri = uplo == 1 ? 1 : 2;
  if (k == 0 || alpha == 0.0) {
    launch_dbeta_tri(m, beta, C, ldc, tri, s);
    return check_cuda(cudaGetLastError(), "gemmt beta");
  }
  return dgemm_select(ta, tb, m, m, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, s);
}

// trans 0: C = alpha A B^T + alpha B A^T + beta C (A, B n x k);
// trans 1: C = alpha A^T B + alpha B^T A + beta C (A, B k x n).
int dsyr2k_device(int uplo, int trans, int64_t n, int64_t k, double alpha, const double *A,
                  int64_t lda, const double *B, int64_t ldb, double beta, double *C, int64_t ldc,
                  cudaStream_t s) {
  if (n == 0) return GB_SUCCESS;
  const int tri = uplo == 1 ? 1 : 2;
  if (k == 0 || alpha == 0.0) {
    launch_dbeta_tri(n, beta, C, ldc, tri, s);
    return check_cuda(cudaGetLastError(), "syr2k beta");
  }
  const int ta = trans ? 1 : 0, tb = trans ? 0 : 1;
  int st = dgemm_select(ta, tb, n, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, s);
  if (st) return st;
  return dgemm_select(ta, tb, n, n, k, alpha, B, ldb, A, lda, 1.0, C, ldc, tri, s);
}

// side 0: B = alpha op(A) B (A m x m); side 1: B = alpha B op(A) (A n x n).
int dtrmm_device(int side, int uplo, int trans, int unit_code, int64_t m, int64_t n,
                 double alpha, const double *A, int64_t lda, double *B, int64_t ldb,
                 cudaStream_t s) {
  if (m == 0 || n == 0) return GB_SUCCESS;
  if (alpha == 0.0) {
    launch_dgemm_beta(m, n, 0.0, B, ldb, s);  // trsm.c/trmm: alpha == 0 zeroes B
    return check_cuda(cudaGetLastError(), "trmm zero");
  }
  const int64_t na = side ? n : m;
  Scratch ws(((size_t)na * na + (size_t)m * n) * sizeof(double), s);
  if (!ws.p) return GB_ERR_ALLOC;
  double *T = ws.as<double>();
  double *Bt = T + na * na;
  const int64_t total = na * na;
  const int64_t blocks = (total + 255) / 256, cap = (int64_t)sm_count() * 16;
  { tri_copy_kernel<<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(na, A, lda, uplo, unit_code, T); count_launch(); }
  GB_CUDA(cudaMemcpy2DAsync(Bt, m * 8, B, ldb * 8, m * 8, n, cudaMemcpyDeviceToDevice, s));
  if (side == 0)
    return dgemm_select(trans, 0, m, n, m, alpha, T, na, Bt, m, 0.0, B, ldb, 0, s);
  return dgemm_select(0, trans, m, n, n, alpha, Bt, m, T, na, 0.0, B, ldb, 0, s);
}

}  // namespace gb
