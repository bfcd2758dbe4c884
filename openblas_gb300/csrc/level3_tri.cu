// Blocked triangular solve (TRSM) and symmetric rank-k update (SYRK).
//
// TRSM follows the structure of driver/level3/trsm_L.c:71-254 and
// trsm_R.c:71-357: B is scaled by alpha first (alpha==0 zeroes B and
// returns); then, walking the diagonal blocks of op(A) in solve order, each
// NB x NB diagonal block is solved against its block row (Left) or block
// column (Right) of B, and the not-yet-solved part of B is updated with a
// GEMM.  The diagonal-block solve multiplies by the reciprocal of the
// diagonal, as the reference's trsm copy routines do (they store 1/a_ii,
// kernel/generic/trsm_ltcopy_4.c).  One thread owns one right-hand-side
// vector (a column of B for Left, a row of B for Right) held in registers;
// the NB x NB block sits in shared memory and is read by broadcast.
//
// SYRK restates driver/level3/syrk_k.c: triangular beta scaling, then the
// GEMM A*A^T (or A^T*A) restricted to the tiles that meet the stored
// triangle, with element-level masking on the diagonal tiles.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_internal.h"

namespace gb {

namespace {

constexpr int TRSM_NB = 32;

// Solve op(Ablk) x = b (left) or x op(Ablk) = b (right) for many vectors.
// Ablk is ib x ib at A (leading dimension lda); vectors are the columns
// (left) or rows (right) of the ib-wide slab of B.  `lower` refers to the
// effective triangle of op(Ablk).
template <typename T, bool LEFT, bool FORWARD>
__global__ void __launch_bounds__(128)
trsm_diag_kernel(int trans, int unit, int ib, int64_t nvec, const T *__restrict__ A,
                 int64_t lda, T *__restrict__ B, int64_t ldb, const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ T Ts[TRSM_NB][TRSM_NB + 1];  // Ts[r][c] = op(Ablk)[r][c]
  __shared__ T inv[TRSM_NB];
  for (int e = threadIdx.x; e < TRSM_NB * TRSM_NB; e += blockDim.x) {
    int r = e % TRSM_NB, c = e / TRSM_NB;
    T v = T(0);
    if (r < ib && c < ib) v = trans ? A[c + (int64_t)r * lda] : A[r + (int64_t)c * lda];
    if (r >= ib && r == c) v = T(1);  // identity padding beyond ib
    Ts[r][c] = v;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < TRSM_NB; r += blockDim.x)
    inv[r] = (unit && r < ib) ? T(1) : T(1) / Ts[r][r];
  __syncthreads();

  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nvec) return;
  // element t of the vector: a column of B (Left) or a row of B (Right)
  T *base = LEFT ? B + v * ldb : B + v;
  const int64_t stride = LEFT ? 1 : ldb;
  T x[TRSM_NB];
#pragma unroll
  for (int t = 0; t < TRSM_NB; ++t) x[t] = (t < ib) ? base[t * stride] : T(0);

  // Left:  T x = b  (column sweep): x_c *= 1/T_cc, then x_r -= T_rc x_c.
  // Right: x T = b  (dot form):     x_c = (b_c - sum_p x_p T_pc) / T_cc.
#pragma unroll
  for (int cc = 0; cc < TRSM_NB; ++cc) {
    const int c = FORWARD ? cc : TRSM_NB - 1 - cc;
    if (LEFT) {
      x[c] *= inv[c];
      if (FORWARD) {
#pragma unroll
        for (int r = c + 1; r < TRSM_NB; ++r) x[r] = fma(-Ts[r][c], x[c], x[r]);
      } else {
#pragma unroll
        for (int r = 0; r < c; ++r) x[r] = fma(-Ts[r][c], x[c], x[r]);
      }
    } else {
      T sacc = x[c];
      if (FORWARD) {
#pragma unroll
        for (int p = 0; p < c; ++p) sacc = fma(-x[p], Ts[p][c], sacc);
      } else {
#pragma unroll
        for (int p = c + 1; p < TRSM_NB; ++p) sacc = fma(-x[p], Ts[p][c], sacc);
      }
      x[c] = sacc * inv[c];
    }
  }
#pragma unroll
  for (int t = 0; t < TRSM_NB; ++t)
    if (t < ib) base[t * stride] = x[t];
}

// The same solves with one warp per vector, lane t holding element t: for
// few vectors (the Cholesky's in-block panels), where one thread per vector
// leaves most SMs idle and runs each vector's ~NB^2/2 FP64 FMAs in series.
// Step c finalises element c (times 1/T_cc) and broadcasts it; the lanes it
// still affects apply their FMA.  Every element sees the same FMAs in the
// same order as in the thread-per-vector kernel (Left: x_r -= T_rc x_c in
// solve order; Right forward: x_c = (b_c - sum_p x_p T_pc) / T_cc with p
// ascending), so the results are the same bit for bit.  Right backward sums
// its dot products with p ascending against a descending solve, so it keeps
// the thread-per-vector kernel.
template <typename T, bool LEFT, bool FORWARD>
__global__ void __launch_bounds__(128)
trsm_diag_warp_kernel(int trans, int unit, int ib, int64_t nvec, const T *__restrict__ A,
                      int64_t lda, T *__restrict__ B, int64_t ldb, const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ T Ts[TRSM_NB][TRSM_NB + 1];  // Ts[r][c] = op(Ablk)[r][c]
  __shared__ T inv[TRSM_NB];
  for (int e = threadIdx.x; e < TRSM_NB * TRSM_NB; e += blockDim.x) {
    int r = e % TRSM_NB, c = e / TRSM_NB;
    T v = T(0);
    if (r < ib && c < ib) v = trans ? A[c + (int64_t)r * lda] : A[r + (int64_t)c * lda];
    if (r >= ib && r == c) v = T(1);
    Ts[r][c] = v;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < TRSM_NB; r += blockDim.x)
    inv[r] = (unit && r < ib) ? T(1) : T(1) / Ts[r][r];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t v = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (v >= nvec) return;  // whole warps leave together
  T *base = LEFT ? B + v * ldb : B + v;
  const int64_t stride = LEFT ? 1 : ldb;
  T x = lane < ib ? base[lane * stride] : T(0);
#pragma unroll
  for (int cc = 0; cc < TRSM_NB; ++cc) {
    const int c = FORWARD ? cc : TRSM_NB - 1 - cc;
    if (lane == c) x *= inv[c];
    const T xc = __shfl_sync(0xffffffffu, x, c);
    const bool later = FORWARD ? lane > c : lane < c;
    if (later) x = LEFT ? fma(-Ts[lane][c], xc, x) : fma(-xc, Ts[c][lane], x);
  }
  if (lane < ib) base[lane * stride] = x;
}

template <typename T>
void launch_trsm_diag(bool left, bool forward, int trans, int unit, int ib, int64_t nvec,
                      const T *A, int64_t lda, T *B, int64_t ldb, cudaStream_t s,
                      const int *skip) {
  if (nvec < 4096 && (left || forward)) {
    const unsigned wgrid = (unsigned)((nvec + 3) / 4);  // four vectors (warps) per block
    if (left && forward)
      { trsm_diag_warp_kernel<T, true, true><<<wgrid, 128, 0, s>>>(trans, unit, ib, nvec, A, lda, B, ldb, skip); count_launch(); }
    else if (left)
      { trsm_diag_warp_kernel<T, true, false><<<wgrid, 128, 0, s>>>(trans, unit, ib, nvec, A, lda, B, ldb, skip); count_launch(); }
    else
      { trsm_diag_warp_kernel<T, false, true><<<wgrid, 128, 0, s>>>(trans, unit, ib, nvec, A, lda, B, ldb, skip); count_launch(); }
    return;
  }
  const unsigned grid = (unsigned)((nvec + 127) / 128);
  if (left && forward)
    { trsm_diag_kernel<T, true, true><<<grid, 128, 0, s>>>(trans, unit, ib, nvec, A, lda, B, ldb, skip); count_launch(); }
  else if (left)
    { trsm_diag_kernel<T, true, false><<<grid, 128, 0, s>>>(trans, unit, ib, nvec, A, lda, B, ldb, skip); count_launch(); }
  else if (forward)
    { trsm_diag_kernel<T, false, true><<<grid, 128, 0, s>>>(trans, unit, ib, nvec, A, lda, B, ldb, skip); count_launch(); }
  else
    { trsm_diag_kernel<T, false, false><<<grid, 128, 0, s>>>(trans, unit, ib, nvec, A, lda, B,
                                                           ldb, skip); count_launch(); }
}

template <typename T>
void gemm_update(int ta, int tb, int64_t m, int64_t n, int64_t k, const T *A, int64_t lda,
                 const T *B, int64_t ldb, T *C, int64_t ldc, cudaStream_t s, const int *skip);
template <>
void gemm_update<double>(int ta, int tb, int64_t m, int64_t n, int64_t k, const double *A,
                         int64_t lda, const double *B, int64_t ldb, double *C, int64_t ldc,
                         cudaStream_t s, const int *skip) {
  launch_dgemm_fp64_tri(ta, tb, m, n, k, -1.0, A, lda, B, ldb, 1.0, C, ldc, 0, s, skip);
}
template <>
void gemm_update<float>(int ta, int tb, int64_t m, int64_t n, int64_t k, const float *A,
                        int64_t lda, const float *B, int64_t ldb, float *C, int64_t ldc,
                        cudaStream_t s, const int *skip) {
  launch_sgemm_fp32_tri(ta, tb, m, n, k, -1.0f, A, lda, B, ldb, 1.0f, C, ldc, 0, s, skip);
}

}  // namespace

// side 0 = Left, 1 = Right; uplo 0 = Upper, 1 = Lower; trans 0/1; unit 0 =
// unit diagonal, 1 = non-unit (the encoding of interface/trsm.c:166-200).
template <typename T>
int trsm_device_t(int side, int uplo, int trans, int unit_code, int64_t m, int64_t n, T alpha,
                  const T *A, int64_t lda, T *B, int64_t ldb, cudaStream_t s,
                  const int *skip = nullptr) {
  if (m == 0 || n == 0) return GB_SUCCESS;
  if (alpha != T(1)) {
    if (sizeof(T) == 8)
      launch_dgemm_beta(m, n, (double)alpha, (double *)B, ldb, s);
    else
      launch_sgemm_beta(m, n, (float)alpha, (float *)B, ldb, s);
    if (alpha == T(0)) return check_cuda(cudaGetLastError(), "trsm alpha scaling");
  }
  const int unit = unit_code == 0;
  const int lower_eff = (uplo == 1) ^ trans;  // triangle of op(A)
  const bool left = side == 0;
  const int64_t na = left ? m : n;
  const int64_t nvec = left ? n : m;
  const int64_t nblk = (na + TRSM_NB - 1) / TRSM_NB;
  // Left: forward when op(A) is lower.  Right: forward when op(A) is upper.
  const bool forward = left ? lower_eff : !lower_eff;
  for (int64_t bi = 0; bi < nblk; ++bi) {
    const int64_t blk = forward ? bi : nblk - 1 - bi;
    const int64_t i0 = blk * TRSM_NB;
    const int ib = (int)((na - i0) < TRSM_NB ? (na - i0) : TRSM_NB);
    const T *Aii = A + i0 + i0 * lda;
    T *Bi = left ? B + i0 : B + i0 * ldb;
    launch_trsm_diag<T>(left, forward, trans, unit, ib, nvec, Aii, lda, Bi, ldb, s, skip);
    // op(A) element (r,c) lives at A[r + c*lda] (no trans) or A[c + r*lda] (trans)
    auto opA = [&](int64_t r, int64_t c) -> const T * {
      return trans ? A + c + r * lda : A + r + c * lda;
    };
    if (left) {
      if (forward && i0 + ib < m) {
        // B[i0+ib:m, :] -= op(A)[i0+ib:m, i0:i0+ib] * B_i
        gemm_update<T>(trans, 0, m - i0 - ib, n, ib, opA(i0 + ib, i0), lda, Bi, ldb,
                       B + i0 + ib, ldb, s, skip);
      } else if (!forward && i0 > 0) {
        // B[0:i0, :] -= op(A)[0:i0, i0:i0+ib] * B_i
        gemm_update<T>(trans, 0, i0, n, ib, opA(0, i0), lda, Bi, ldb, B, ldb, s, skip);
      }
    } else {
      if (forward && i0 + ib < n) {
        // B[:, i0+ib:n] -= X_i * op(A)[i0:i0+ib, i0+ib:n]
        gemm_update<T>(0, trans, m, n - i0 - ib, ib, Bi, ldb, opA(i0, i0 + ib), lda,
                       B + (i0 + ib) * ldb, ldb, s, skip);
      } else if (!forward && i0 > 0) {
        // B[:, 0:i0] -= X_i * op(A)[i0:i0+ib, 0:i0]
        gemm_update<T>(0, trans, m, i0, ib, Bi, ldb, opA(i0, 0), lda, B, ldb, s, skip);
      }
    }
  }
  return check_cuda(cudaGetLastError(), "trsm launch");
}

int dtrsm_device(int side, int uplo, int trans, int unit, int64_t m, int64_t n, double alpha,
                 const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s) {
  return trsm_device_t<double>(side, uplo, trans, unit, m, n, alpha, A, lda, B, ldb, s);
}

namespace {
// Leaves of the recursive emulated-FP64 TRSM: solved by the native blocked
// TRSM above.
constexpr int64_t TRSM_EMU_LEAF = 128;

// Solve for the triangular index range [i0, i0 + len) of op(A) (rows of B on
// the left, columns on the right): halves in the order of the substitution,
// the later half updated with the solved one by one FP64-accurate GEMM
// (X1 = op(A11)^-1 B1, B2 -= op(A21) X1, X2 = op(A22)^-1 B2, as
// driver/level3/trsm_L.c's blocked loop does with GEMM_P blocks).
int trsm_rec_emulated(int side, int uplo, int trans, int unit_code, int64_t m, int64_t n,
                      const double *A, int64_t lda, double *B, int64_t ldb, bool forward,
                      int64_t i0, int64_t len, cudaStream_t s) {
  const bool left = side == 0;
  if (len <= TRSM_EMU_LEAF)
    return trsm_device_t<double>(side, uplo, trans, unit_code, left ? len : m, left ? n : len,
                                 1.0, A + i0 + i0 * lda, lda, left ? B + i0 : B + i0 * ldb, ldb,
                                 s);
  // first half, a multiple of 128 (and shorter than len: len > 256)
  int64_t h = (len / 2 + 127) / 128 * 128;
  if (h >= len) h = len / 2;
  const int64_t f0 = forward ? i0 : i0 + len - h, fl = h;
  const int64_t s0 = forward ? i0 + h : i0, sl = len - h;
  auto opA = [&](int64_t r, int64_t c) { return trans ? A + c + r * lda : A + r + c * lda; };
  int st = trsm_rec_emulated(side, uplo, trans, unit_code, m, n, A, lda, B, ldb, forward, f0, fl,
                             s);
  if (st) return st;
  // the caller's slice setting, as for DGEMM (automatic: per-tile tolerance)
  const int slices = ozaki_caller_slices();
  if (left)
    st = dgemm_emulated(trans, 0, sl, n, fl, -1.0, opA(s0, f0), lda, B + f0, ldb, 1.0, B + s0,
                        ldb, slices, s);
  else
    st = dgemm_emulated(0, trans, m, sl, fl, -1.0, B + f0 * ldb, ldb, opA(f0, s0), lda, 1.0,
                        B + s0 * ldb, ldb, slices, s);
  if (st) return st;
  return trsm_rec_emulated(side, uplo, trans, unit_code, m, n, A, lda, B, ldb, forward, s0, sl,
                           s);
}
}  // namespace

// The caller-facing DTRSM (dtrsm_, cblas_dtrsm, gb_dtrsm_dev): with the
// emulated-FP64 DGEMM selected (or in auto mode for a large solve) and a
// triangle wider than one leaf, the recursive form above moves all but the
// leaves' 128-wide diagonal solves onto the tensor cores; otherwise the
// native blocked TRSM.
int dtrsm_select(int side, int uplo, int trans, int unit, int64_t m, int64_t n, double alpha,
                 const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s) {
  const bool left = side == 0;
  const int64_t na = left ? m : n, nvec = left ? n : m;
  const int mode = gb_get_dgemm_mode();
  const bool emulated =
      mode == GB_DGEMM_EMULATED ||
      (mode == GB_DGEMM_AUTO && (double)na * na * nvec >= 512.0 * 512.0 * 512.0);
  if (!emulated || na <= TRSM_EMU_LEAF || m == 0 || n == 0 || alpha == 0.0)
    return dtrsm_device(side, uplo, trans, unit, m, n, alpha, A, lda, B, ldb, s);
  if (alpha != 1.0) launch_dgemm_beta(m, n, alpha, B, ldb, s);
  const int lower_eff = (uplo == 1) ^ trans;  // triangle of op(A)
  const bool forward = left ? lower_eff : !lower_eff;
  return trsm_rec_emulated(side, uplo, trans, unit, m, n, A, lda, B, ldb, forward, 0, na, s);
}

int dtrsm_device_skip(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                      double alpha, const double *A, int64_t lda, double *B, int64_t ldb,
                      cudaStream_t s, const int *skip) {
  return trsm_device_t<double>(side, uplo, trans, unit, m, n, alpha, A, lda, B, ldb, s, skip);
}

int strsm_device(int side, int uplo, int trans, int unit, int64_t m, int64_t n, float alpha,
                 const float *A, int64_t lda, float *B, int64_t ldb, cudaStream_t s) {
  return trsm_device_t<float>(side, uplo, trans, unit, m, n, alpha, A, lda, B, ldb, s);
}

int strsm_device_skip(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                      float alpha, const float *A, int64_t lda, float *B, int64_t ldb,
                      cudaStream_t s, const int *skip) {
  return trsm_device_t<float>(side, uplo, trans, unit, m, n, alpha, A, lda, B, ldb, s, skip);
}

int ssyrk_device_skip(int uplo, int trans, int64_t n, int64_t k, float alpha, const float *A,
                      int64_t lda, float beta, float *C, int64_t ldc, cudaStream_t s,
                      const int *skip) {
  if (n == 0) return GB_SUCCESS;
  launch_sgemm_fp32_tri(trans ? 1 : 0, trans ? 0 : 1, n, n, k, alpha, A, lda, A, lda, beta, C,
                        ldc, uplo == 1 ? 1 : 2, s, skip);
  return check_cuda(cudaGetLastError(), "syrk launch");
}

// uplo 0 = Upper, 1 = Lower; trans 0: C = alpha*A*A^T + beta*C (A n x k),
// trans 1: C = alpha*A^T*A + beta*C (A k x n).
int dsyrk_device_skip(int uplo, int trans, int64_t n, int64_t k, double alpha, const double *A,
                      int64_t lda, double beta, double *C, int64_t ldc, cudaStream_t s,
                      const int *skip) {
  if (n == 0) return GB_SUCCESS;
  launch_dgemm_fp64_tri(trans ? 1 : 0, trans ? 0 : 1, n, n, k, alpha, A, lda, A, lda, beta, C,
                        ldc, uplo == 1 ? 1 : 2, s, skip);
  return check_cuda(cudaGetLastError(), "syrk launch");
}

// The caller-facing DSYRK: the stored triangle of alpha op(A) op(A)^T + beta C
// with the FP64 GEMM the DGEMM mode selects (tiles outside the triangle
// skipped).
int dsyrk_device(int uplo, int trans, int64_t n, int64_t k, double alpha, const double *A,
                 int64_t lda, double beta, double *C, int64_t ldc, cudaStream_t s) {
  if (n == 0) return GB_SUCCESS;
  const int tri = uplo == 1 ? 1 : 2;
  if (k == 0 || alpha == 0.0) {
    launch_dbeta_tri(n, beta, C, ldc, tri, s);
    return check_cuda(cudaGetLastError(), "syrk launch");
  }
  return dgemm_select(trans ? 1 : 0, trans ? 0 : 1, n, n, k, alpha, A, lda, A, lda, beta, C, ldc,
                      tri, s);
}

}  // namespace gb
