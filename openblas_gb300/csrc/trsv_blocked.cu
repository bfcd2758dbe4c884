// LU solve for a few right-hand sides with inverted diagonal blocks.
//
// getrs (lapack/getrs/getrs_single.c:42-68) applies the interchanges and two
// triangular solves; for one right-hand side the reference switches to TRSV
// (driver/level2/trsv_L.c, trsv_U.c), a latency-bound sweep.  Here the
// diagonal blocks (TB x TB) of the unit-lower L and of U are inverted once
// per factorisation; each solve step i is then one kernel in which every CTA
// recomputes x_i = inv(D_ii) * b_i (a small dense product, no inter-CTA
// dependency) and updates its share of the remaining rows,
// b_r -= A_{r,i} x_i.  A solve is n/TB launches that read the triangle once.
// Used by the mixed-precision solver's refinement steps, where the factors
// are reused many times.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_internal.h"
#include "lapack_internal.h"

namespace gb {

namespace {

constexpr int TB = 64;           // diagonal block size
// right-hand sides per solve pass (static shared memory stays within 48 KB)
template <typename T>
constexpr int maxr() { return sizeof(T) == 4 ? 32 : 16; }

// Inverse of the diagonal block of L (unit lower, lower = 1) or U (upper,
// lower = 0).  One CTA per block, thread c computes column c of the inverse
// by substitution on e_c.  Blocks shorter than TB are padded with identity.
template <typename T>
__global__ void __launch_bounds__(TB)
diag_inverse_kernel(int64_t n, const T *__restrict__ A, int64_t lda, int lower,
                    T *__restrict__ inv) {
  __shared__ T D[TB][TB + 1];
  const int64_t b = blockIdx.x;
  const int64_t r0 = b * TB;
  const int nb = (int)((n - r0) < TB ? (n - r0) : TB);
  for (int e = threadIdx.x; e < TB * TB; e += TB) {
    const int r = e % TB, c = e / TB;
    T v = T(0);
    if (r < nb && c < nb) v = A[(r0 + r) + (r0 + c) * lda];
    if (r == c && (r >= nb || lower)) v = T(1);  // unit diagonal of L, identity padding
    D[r][c] = v;
  }
  __syncthreads();
  const int c = threadIdx.x;
  T x[TB];
#pragma unroll
  for (int r = 0; r < TB; ++r) x[r] = (r == c) ? T(1) : T(0);
  if (lower) {
#pragma unroll
    for (int r = 0; r < TB; ++r) {
      T s = x[r];
#pragma unroll
      for (int k = 0; k < r; ++k) s = fma(-D[r][k], x[k], s);
      x[r] = s;  // unit diagonal
    }
  } else {
#pragma unroll
    for (int rr = 0; rr < TB; ++rr) {
      const int r = TB - 1 - rr;
      T s = x[r];
#pragma unroll
      for (int k = r + 1; k < TB; ++k) s = fma(-D[r][k], x[k], s);
      x[r] = s / D[r][r];
    }
  }
  T *out = inv + b * (TB * TB);  // column-major TB x TB
#pragma unroll
  for (int r = 0; r < TB; ++r) out[r + c * TB] = x[r];
}

// One step of the blocked solve: x_i = inv_i * w_i (every CTA computes it
// from the working buffer W, whose block i no step of this pass writes),
// CTA 0 stores x_i into the output buffer X, and rows [u0, u1) of W get
// w_r -= A(r, block i) x_i.
template <typename T, int R>
__global__ void __launch_bounds__(256)
block_solve_step_kernel(int nrhs, const T *__restrict__ A, int64_t lda,
                        const T *__restrict__ inv, int64_t r0, int nb, T *__restrict__ W,
                        int64_t ldw, T *__restrict__ X, int64_t ldx, int64_t u0, int64_t u1) {
  __shared__ T Iv[TB * TB];  // inverted diagonal block, column-major
  __shared__ T bi[R][TB];
  __shared__ T xi[R][TB];
  const int tid = threadIdx.x;
  const T *src = inv + (r0 / TB) * (TB * TB);
  for (int e = tid; e < TB * TB; e += 256) Iv[e] = src[e];
  for (int e = tid; e < R * TB; e += 256) {
    const int k = e / TB, r = e % TB;
    bi[k][r] = (k < nrhs && r < nb) ? W[(r0 + r) + k * ldw] : T(0);
  }
  __syncthreads();
  for (int e = tid; e < R * TB; e += 256) {
    const int k = e / TB, r = e % TB;
    T s = T(0);
    if (k < nrhs) {
#pragma unroll 16
      for (int c = 0; c < TB; ++c) s = fma(Iv[r + c * TB], bi[k][c], s);
    }
    xi[k][r] = s;
  }
  __syncthreads();
  if (blockIdx.x == 0)
    for (int e = tid; e < nrhs * TB; e += 256) {
      const int k = e / TB, r = e % TB;
      if (r < nb) X[(r0 + r) + k * ldx] = xi[k][r];
    }
  const int64_t rows = u1 - u0;
  for (int64_t rr = (int64_t)blockIdx.x * 256 + tid; rr < rows; rr += (int64_t)gridDim.x * 256) {
    const int64_t r = u0 + rr;
    const T *a = A + r + r0 * lda;
    T acc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) acc[k] = T(0);
    if (nb == TB) {
#pragma unroll 8
      for (int c = 0; c < TB; ++c) {
        const T av = a[c * lda];
#pragma unroll
        for (int k = 0; k < R; ++k) acc[k] = fma(av, xi[k][c], acc[k]);
      }
    } else {
      for (int c = 0; c < nb; ++c) {
        const T av = a[c * lda];
#pragma unroll
        for (int k = 0; k < R; ++k) acc[k] = fma(av, xi[k][c], acc[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (k < nrhs) W[r + k * ldw] -= acc[k];
  }
}

}  // namespace

template <typename T>
int lu_block_inverses(int64_t n, const T *A, int64_t lda, T *Linv, T *Uinv, cudaStream_t s) {
  const unsigned nblk = (unsigned)((n + TB - 1) / TB);
  { diag_inverse_kernel<T><<<nblk, TB, 0, s>>>(n, A, lda, 1, Linv); count_launch(); }
  { diag_inverse_kernel<T><<<nblk, TB, 0, s>>>(n, A, lda, 0, Uinv); count_launch(); }
  return check_cuda(cudaGetLastError(), "diag_inverse");
}

// Solve L U X = B in place (interchanges already applied), in passes of
// MAXR columns.  The forward pass works in B and writes y to the scratch Y;
// the backward pass works in Y and writes x back into B.
template <typename T>
int lu_block_solve(int64_t n, int64_t nrhs, const T *A, int64_t lda, const T *Linv,
                   const T *Uinv, T *B, int64_t ldb, cudaStream_t s) {
  const int64_t nblk = (n + TB - 1) / TB;
  constexpr int MAXR = maxr<T>();
  Scratch ws((size_t)n * MAXR * sizeof(T), s);
  if (!ws.p) return GB_ERR_ALLOC;
  T *Y = ws.as<T>();
  auto grid = [&](int64_t rows) {
    int64_t g = (rows + 255) / 256;
    if (g < 1) g = 1;
    if (g > (int64_t)sm_count() * 4) g = (int64_t)sm_count() * 4;
    return (unsigned)g;
  };
  for (int64_t k0 = 0; k0 < nrhs; k0 += MAXR) {
    const int kk = (int)((nrhs - k0) < MAXR ? (nrhs - k0) : MAXR);
    T *Bk = B + k0 * ldb;
    auto step = [&](const T *inv, int64_t r0, int nb, T *Wb, int64_t ldw, T *Xb, int64_t ldx,
                    int64_t u0, int64_t u1) {
      const unsigned g = grid(u1 - u0);
      if (kk <= 4)
        block_solve_step_kernel<T, 4><<<g, 256, 0, s>>>(kk, A, lda, inv, r0, nb, Wb, ldw, Xb, ldx, u0, u1);
      else
        block_solve_step_kernel<T, MAXR><<<g, 256, 0, s>>>(kk, A, lda, inv, r0, nb, Wb, ldw, Xb, ldx, u0, u1);
      count_launch();
    };
    for (int64_t i = 0; i < nblk; ++i) {  // forward: L y = b
      const int64_t r0 = i * TB;
      const int nb = (int)((n - r0) < TB ? (n - r0) : TB);
      step(Linv, r0, nb, Bk, ldb, Y, n, r0 + nb, n);
    }
    for (int64_t i = nblk - 1; i >= 0; --i) {  // backward: U x = y
      const int64_t r0 = i * TB;
      const int nb = (int)((n - r0) < TB ? (n - r0) : TB);
      step(Uinv, r0, nb, Y, n, Bk, ldb, 0, r0);
    }
  }
  return check_cuda(cudaGetLastError(), "lu_block_solve");
}

template int lu_block_inverses<float>(int64_t, const float *, int64_t, float *, float *,
                                      cudaStream_t);
template int lu_block_inverses<double>(int64_t, const double *, int64_t, double *, double *,
                                       cudaStream_t);
template int lu_block_solve<float>(int64_t, int64_t, const float *, int64_t, const float *,
                                   const float *, float *, int64_t, cudaStream_t);
template int lu_block_solve<double>(int64_t, int64_t, const double *, int64_t, const double *,
                                    const double *, double *, int64_t, cudaStream_t);

}  // namespace gb
