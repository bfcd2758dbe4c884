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
// Leaves of the recursive emulated-FP64 TRSM: triangles of at most 128.
constexpr int64_t TRSM_EMU_LEAF = 128;

// One leaf in one launch: a whole triangle of nb <= 128 columns against 32
// right-hand-side vectors per CTA.  The blocked path above spends four
// diagonal-block launches (64 CTAs of 128 vectors at 8192 vectors) and three
// FP64 GEMMs of depth 32 on it, which keeps the FP64 pipe, the scarcest unit
// on this part, about half busy.  The solve is the column sweep of the
// substitution, walked in 32-wide blocks as driver/level3/trsm_L.c walks its
// GEMM_P blocks: element c takes x_c *= 1/T_cc, then every later element r
// takes x_r -= T_rc x_c, c ascending.  The 32 vectors (columns of B on the
// left, rows on the right) sit in shared memory, 128 x 32 doubles with an
// XOR swizzle, so the coalesced loads along a vector and the one-thread-per-
// vector accesses both meet the two-wavefront minimum; the triangle is
// staged 32 columns at a time and read by broadcast.  The four warps share
// each diagonal block's solve (rows dealt round robin, one barrier per
// column) and then update the later rows in groups of four (four
// independent FMA chains per thread).  Each SM sub-partition's FP64 unit
// takes about 64 clocks per warp-wide DFMA, so all four warps must carry
// FP64 work at every phase.
//
// Working order: element i of the working vector is element o(i) of the
// stored one, o(i) = i (FORWARD) or nb - 1 - i, so the working triangle
// L'[i][j] = Leff[o(i)][o(j)] is lower.  Leff = op(A) on the left and
// op(A)^T on the right (x op(A) = b is op(A)^T x^T = b^T); with
// eff_t = trans ^ right, Leff[r][c] = A[r + c lda] (eff_t 0) or A[c + r lda].
constexpr int LEAF_V = 32;        // vectors per CTA, one per lane
constexpr int LEAF_THREADS = 128;
constexpr int LEAF_PLD = 33;      // row pitch of the staged panel (doubles)
constexpr size_t LEAF_SMEM =
    sizeof(double) * ((size_t)TRSM_EMU_LEAF * LEAF_V + (size_t)TRSM_EMU_LEAF * LEAF_PLD + 32);

template <bool FORWARD>
__global__ void __launch_bounds__(LEAF_THREADS)
trsm_leaf_kernel(int right, int eff_t, int unit, int nb, int64_t nvec,
                 const double *__restrict__ A, int64_t lda, double *__restrict__ B,
                 int64_t ldb) {
  constexpr int NBMAX = (int)TRSM_EMU_LEAF;
  extern __shared__ double leaf_smem[];
  double *Xs = leaf_smem;                // [NBMAX][LEAF_V], swizzled columns
  double *Ps = Xs + NBMAX * LEAF_V;      // [NBMAX][LEAF_PLD]: rows j0.. of the panel
  double *inv = Ps + NBMAX * LEAF_PLD;   // [32]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t v0 = (int64_t)blockIdx.x * LEAF_V;
  const int nv = (int)(nvec - v0 < LEAF_V ? nvec - v0 : LEAF_V);
  auto xs = [&](int i, int v) -> double & { return Xs[i * LEAF_V + (v ^ (i & 31))]; };
  auto o = [&](int i) { return FORWARD ? i : nb - 1 - i; };

  // the vectors, element o(i) at working row i (zero beyond nb and nv)
  if (!right) {
#pragma unroll 4
    for (int v = warp; v < LEAF_V; v += 4)
      for (int i = lane; i < NBMAX; i += 32)
        xs(i, v) = (v < nv && i < nb) ? B[o(i) + (v0 + v) * ldb] : 0.0;
  } else {
#pragma unroll 4
    for (int i = warp; i < NBMAX; i += 4)
      xs(i, lane) = (lane < nv && i < nb) ? B[v0 + lane + (int64_t)o(i) * ldb] : 0.0;
  }

  for (int j0 = 0; j0 < nb; j0 += 32) {
    const int cb = nb - j0 < 32 ? nb - j0 : 32;
    __syncthreads();  // the previous block's panel reads and row updates are done
    // panel: Ps[(i - j0) * LEAF_PLD + jj] = L'[i][j0 + jj], i in [j0, nb), jj < cb
    if (eff_t == 0) {
      for (int jj = warp; jj < cb; jj += 4) {
        const double *col = A + (int64_t)o(j0 + jj) * lda;
        for (int i = j0 + lane; i < nb; i += 32) Ps[(i - j0) * LEAF_PLD + jj] = col[o(i)];
      }
    } else {
      for (int i = j0 + warp; i < nb; i += 4)
        if (lane < cb) Ps[(i - j0) * LEAF_PLD + lane] = A[o(j0 + lane) + (int64_t)o(i) * lda];
    }
    if (tid < cb) {
      const int64_t d = o(j0 + tid);
      inv[tid] = unit ? 1.0 : 1.0 / A[d + d * lda];
    }
    __syncthreads();
    {
      // diagonal block over the four warps (one warp alone would leave three
      // of the SM's four FP64 units idle): warp w owns rows w + 4t; at step
      // c the owner of row c scales it by 1/T_cc and publishes it in Xs, and
      // after the barrier every warp applies it to its later rows
      double xr[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int r = warp + 4 * t;
        xr[t] = r < cb ? xs(j0 + r, lane) : 0.0;
      }
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        if (c < cb) {
          if (warp == (c & 3)) {
            xr[c >> 2] *= inv[c];
            xs(j0 + c, lane) = xr[c >> 2];
          }
          __syncthreads();
          const double xc = xs(j0 + c, lane);
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int r = warp + 4 * t;
            if (r > c && r < cb) xr[t] = fma(-Ps[r * LEAF_PLD + c], xc, xr[t]);
          }
        }
      }
    }
    const int r0 = j0 + 32;
    if (r0 >= nb) break;  // the last block (the only one with cb < 32): no later rows
    // every row of the block was published before one of the barriers above
    double x[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) x[c] = xs(j0 + c, lane);
    // rows r0.. in groups of four, the k-th group to warp k % 4; the lanes of
    // a short last group repeat row g and do not store it
    for (int g = r0 + 4 * warp; g < nb; g += 16) {
      const int nr = nb - g < 4 ? nb - g : 4;
      double acc[4];
      const double *prow[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = q < nr ? g + q : g;
        acc[q] = xs(i, lane);
        prow[q] = Ps + (i - j0) * LEAF_PLD;
      }
#pragma unroll
      for (int c = 0; c < 32; ++c) {
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = fma(-prow[q][c], x[c], acc[q]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q < nr) xs(g + q, lane) = acc[q];
    }
  }
  __syncthreads();
  if (!right) {
#pragma unroll 4
    for (int v = warp; v < LEAF_V; v += 4)
      for (int i = lane; i < NBMAX; i += 32)
        if (v < nv && i < nb) B[o(i) + (v0 + v) * ldb] = xs(i, v);
  } else {
#pragma unroll 4
    for (int i = warp; i < NBMAX; i += 4)
      if (lane < nv && i < nb) B[v0 + lane + (int64_t)o(i) * ldb] = xs(i, lane);
  }
}

// The leaf solve op(A) X = B (left, nb = m) or X op(A) = B (right, nb = n),
// nb <= 128, alpha already applied; forward as in trsm_device_t.
int trsm_leaf(bool left, bool forward, int trans, int unit_code, int64_t nb, int64_t nvec,
              const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s) {
  static PerDeviceOnce attr_once;
  const int ast = attr_once.run(current_device(), [] {
    GB_CUDA(cudaFuncSetAttribute(trsm_leaf_kernel<true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LEAF_SMEM));
    GB_CUDA(cudaFuncSetAttribute(trsm_leaf_kernel<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LEAF_SMEM));
    return GB_SUCCESS;
  });
  if (ast) return ast;
  const int right = left ? 0 : 1, eff_t = trans ^ right, unit = unit_code == 0;
  const unsigned grid = (unsigned)((nvec + LEAF_V - 1) / LEAF_V);
  if (forward)
    { trsm_leaf_kernel<true><<<grid, LEAF_THREADS, LEAF_SMEM, s>>>(right, eff_t, unit, (int)nb, nvec, A, lda, B, ldb); count_launch(); }
  else
    { trsm_leaf_kernel<false><<<grid, LEAF_THREADS, LEAF_SMEM, s>>>(right, eff_t, unit, (int)nb, nvec, A, lda, B, ldb); count_launch(); }
  return check_cuda(cudaGetLastError(), "trsm leaf");
}

// Solve for the triangular index range [i0, i0 + len) of op(A) (rows of B on
// the left, columns on the right): halves in the order of the substitution,
// the later half updated with the solved one by one FP64-accurate GEMM
// (X1 = op(A11)^-1 B1, B2 -= op(A21) X1, X2 = op(A22)^-1 B2, as
// driver/level3/trsm_L.c's blocked loop does with GEMM_P blocks).
int trsm_rec_emulated(int side, int uplo, int trans, int unit_code, int64_t m, int64_t n,
                      const double *A, int64_t lda, double *B, int64_t ldb, bool forward,
                      int64_t i0, int64_t len, cudaStream_t s) {
  const bool left = side == 0;
  if (len <= TRSM_EMU_LEAF) {
    ProfileScope prof("trsm_leaf", s);
    return trsm_leaf(left, forward, trans, unit_code, len, left ? n : m, A + i0 + i0 * lda, lda,
                     left ? B + i0 : B + i0 * ldb, ldb, s);
  }
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
  {
    ProfileScope prof("trsm_emu_gemm", s);
    if (left)
      st = dgemm_emulated(trans, 0, sl, n, fl, -1.0, opA(s0, f0), lda, B + f0, ldb, 1.0, B + s0,
                          ldb, slices, s);
    else
      st = dgemm_emulated(0, trans, m, sl, fl, -1.0, B + f0 * ldb, ldb, opA(f0, s0), lda, 1.0,
                          B + s0 * ldb, ldb, slices, s);
  }
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
