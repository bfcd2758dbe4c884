// Grouped batches of small uneven problems in one persistent launch.
//
// The reference runs cblas_dgemm_batch (interface/gemm_batch.c:117-372,
// driver/level3/gemm_batch_thread.c:79-156) by looping over the problems or
// handing chunks of them to its threads; it has no batched LU/Cholesky.  Here
// a device-side problem table (DGEMM, DGESV = DGETRF+DGETRS, DPOTRF) is
// processed by one persistent kernel: every CTA takes the next problem from
// an atomic counter over a list sorted by decreasing cost, so uneven sizes
// balance across the SMs.  A plan uploads the table once, autotunes the CTA
// size on the actual batch (the choice is cached under a key made of the
// problem-size histogram), and captures the launch in a CUDA graph that is
// replayed for every execution.
//
// Per-problem algorithms (one CTA each; FP64 throughput bounds these sizes
// on this part, so each is arranged to keep the FP64 pipe busy):
//   DGEMM   C = alpha op(A) op(B) + beta C, register-tiled CTA loop over
//           64x64 or 32x32 tiles of C (the tile per size bin is picked by the
//           autotuner: small problems waste less padding on 32x32 tiles);
//           beta == 0 overwrites C (gemm_beta.c:41-94).
//   DGESV   blocked right-looking LU (lapack/getrf/getrf_single.c structure,
//           16-column panels): each panel is factored in shared memory with
//           the getf2_k.c pivot rules (first maximum |a|, swap of the panel's
//           processed columns and reciprocal scaling only when |pivot| >=
//           DBL_MIN, info = first zero pivot), its interchanges go to the
//           columns on both sides (laswp), then U12 and the trailing matrix
//           are updated once per panel, every element taking the panel's
//           multipliers in column order (the arithmetic of the column-by-column
//           rank-1 updates, read and written once per panel instead of once per
//           column); then forward/back substitution of the right-hand sides
//           when info == 0 (gesv.c:131-135).
//           Mixed variant: the LU runs in FP32 on a scratch copy, the solution
//           is refined in FP64 with the dsgesv.f stopping test; problems that
//           do not converge in 30 steps are redone in FP64 by the same CTA.
//   DPOTRF  blocked right-looking Cholesky, 16-column panels in shared memory
//           (potf2_L.c / potf2_U.c contract: info = first non-positive pivot,
//           whose value is left in place; columns before it are final and the
//           rest carries the updates of those columns).
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gb_internal.h"
#include "operand.h"
#include "ozaki_digits.cuh"
#include <cuda_bf16.h>

namespace gb {

namespace {

struct DevProblem {
  int type, m, n, k;
  int ta, tb, uplo, tile;  // tile: DGEMM tile edge (32 or 64)
  double alpha, beta;
  void *A, *B, *C;
  int lda, ldb, ldc, pad2;
  int *info;
  float *work;  // FP32 scratch for the mixed DGESV variant (n*n + 2n floats)
};

// ---------------------------------------------------------------- DGEMM
constexpr int DG_BK = 16;
constexpr int PANEL_B = 16;  // panel width of the blocked LU and Cholesky
constexpr int TILE_BINS = 4; // size bins of the DGEMM tile choice

template <int NT, int BM>
__device__ void cta_dgemm(const DevProblem &p, double *smem) {
  constexpr int BN = BM, BK = DG_BK;
  constexpr int TX = 16, TY = NT / TX;  // thread grid over the tile
  static_assert(BM % TX == 0 && BN % TY == 0 && TX * TY == NT, "tile split");
  constexpr int RM = BM / TX, RN = BN / TY;
  double(*As)[BM] = reinterpret_cast<double(*)[BM]>(smem);
  double(*Bs)[BN] = reinterpret_cast<double(*)[BN]>(smem + BK * BM);
  const double *A = (const double *)p.A, *B = (const double *)p.B;
  double *C = (double *)p.C;
  const int m = p.m, n = p.n, k = p.k;
  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
  for (int m0 = 0; m0 < m; m0 += BM)
    for (int n0 = 0; n0 < n; n0 += BN) {
      double acc[RM][RN];
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < RN; ++j) acc[i][j] = 0.0;
      if (p.alpha != 0.0)
        for (int k0 = 0; k0 < k; k0 += BK) {
          __syncthreads();
          for (int e = tid; e < BM * BK; e += NT) {
            int i, kk;
            if (!p.ta) { i = e % BM; kk = e / BM; } else { kk = e % BK; i = e / BK; }
            const int gi = m0 + i, gk = k0 + kk;
            double v = 0.0;
            if (gi < m && gk < k) v = p.ta ? A[gk + (int64_t)gi * p.lda] : A[gi + (int64_t)gk * p.lda];
            As[kk][i] = v;
          }
          for (int e = tid; e < BN * BK; e += NT) {
            int j, kk;
            if (!p.tb) { kk = e % BK; j = e / BK; } else { j = e % BN; kk = e / BN; }
            const int gj = n0 + j, gk = k0 + kk;
            double v = 0.0;
            if (gj < n && gk < k) v = p.tb ? B[gj + (int64_t)gk * p.ldb] : B[gk + (int64_t)gj * p.ldb];
            Bs[kk][j] = v;
          }
          __syncthreads();
#pragma unroll
          for (int kk = 0; kk < BK; ++kk) {
            double a[RM], b[RN];
#pragma unroll
            for (int i = 0; i < RM; ++i) a[i] = As[kk][tx + i * TX];
#pragma unroll
            for (int j = 0; j < RN; ++j) b[j] = Bs[kk][ty + j * TY];
#pragma unroll
            for (int i = 0; i < RM; ++i)
#pragma unroll
              for (int j = 0; j < RN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
          }
        }
#pragma unroll
      for (int j = 0; j < RN; ++j) {
        const int gj = n0 + ty + j * TY;
        if (gj >= n) continue;
#pragma unroll
        for (int i = 0; i < RM; ++i) {
          const int gi = m0 + tx + i * TX;
          if (gi >= m) continue;
          double *c = C + gi + (int64_t)gj * p.ldc;
          double v = p.alpha * acc[i][j];
          *c = (p.beta == 0.0) ? v : fma(p.beta, *c, v);
        }
      }
    }
}

// ---------------------------------------------------------------- DGEMM, emulated FP64
// The Ozaki split of the large-product engine (ozaki.cu) for one small
// problem per CTA, on the warp-level bf16 tensor-core MMA: per 32 x 32 tile
// of C (eight warps of 16 x 8), the rows of op(A) and the columns of op(B) get their scale exponents
// over the whole K; every 64-deep K chunk is cut into EM_S = 7 slices of
// 8-bit digits (56 bits) in shared memory; each product of digit slices
// A_s B_t with s + t <= 8 (the Ozaki triangle, 28 products) is summed by
// mma.sync m16n8k16 in FP32, exact for one chunk (64 * 255^2 < 2^24), and
// added to the int32 sum of its level s + t (at most 7 products x 64 chunks
// x 64 * 255^2 < 2^31 for K <= 4096); the levels are recombined as an exact
// int128 and rounded once (ozd::level_value).  The exponents are found once
// per problem.  Tiles whose rows or columns hold Inf/NaN, K > 4096 and m or n
// above 2048 use the FP64 loop instead.
constexpr int EM_BM = 32, EM_KC = 64, EM_S = 7, EM_KP = 72;  // KP: padded row of a slice
constexpr int EM_NT = 256;
constexpr int EM_KMAX = 4096;
constexpr int EM_DMAX = 2048;  // rows of op(A) / columns of op(B) whose exponents are kept
constexpr size_t EM_SLICE_ELEMS = (size_t)EM_S * EM_BM * EM_KP;
constexpr size_t EM_SMEM = 2 * EM_SLICE_ELEMS * sizeof(__nv_bfloat16) + 2 * EM_DMAX * sizeof(int) + 16;

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4],
                                               uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// FP64 loop for one tile (Inf/NaN present, or K too long for exact levels)
__device__ void emu_tile_fp64(const DevProblem &p, int m0, int n0) {
  const double *A = (const double *)p.A, *B = (const double *)p.B;
  double *C = (double *)p.C;
  for (int e = threadIdx.x; e < EM_BM * EM_BM; e += EM_NT) {
    const int i = m0 + e % EM_BM, j = n0 + e / EM_BM;
    if (i >= p.m || j >= p.n) continue;
    double sum = 0.0;
    if (p.alpha != 0.0)
      for (int k = 0; k < p.k; ++k) {
        const double a = p.ta ? A[k + (int64_t)i * p.lda] : A[i + (int64_t)k * p.lda];
        const double b = p.tb ? B[j + (int64_t)k * p.ldb] : B[k + (int64_t)j * p.ldb];
        sum = fma(a, b, sum);
      }
    double *c = C + i + (int64_t)j * p.ldc;
    const double v = p.alpha * sum;
    *c = (p.beta == 0.0) ? v : fma(p.beta, *c, v);
  }
}

__device__ void cta_dgemm_emu(const DevProblem &p, unsigned char *smem) {
  using namespace ozd;
  __nv_bfloat16 *As = reinterpret_cast<__nv_bfloat16 *>(smem);  // [S][BM][KP]
  __nv_bfloat16 *Bs = As + EM_SLICE_ELEMS;                        // [S][BN][KP]
  int *e_row = reinterpret_cast<int *>(Bs + EM_SLICE_ELEMS);      // [m] exponents of op(A) rows
  int *f_col = e_row + EM_DMAX;                                   // [n] of op(B) columns
  __shared__ int s_special;
  const double *A = (const double *)p.A, *B = (const double *)p.B;
  double *C = (double *)p.C;
  const int m = p.m, n = p.n, k = p.k;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, tg = lane & 3;
  const int wm = (warp & 1) * 16, wn = (warp >> 1) * 8;  // warp's 16 x 8 sub-tile
  const bool fp64 = p.alpha == 0.0 || k == 0 || k > EM_KMAX || m > EM_DMAX || n > EM_DMAX;
  if (!fp64) {
    // scale exponents of every row of op(A) and column of op(B), once: a
    // warp per row or column, its lanes along K (coalesced when the K
    // direction is contiguous; otherwise lanes of neighbouring warps read
    // neighbouring rows of the same column)
    for (int r = warp; r < m + n; r += EM_NT / 32) {
      const bool row = r < m;
      const int rr = row ? r : r - m;
      unsigned long long best = 0;
      for (int kk = lane; kk < k; kk += 32) {
        const double v = row ? (p.ta ? A[kk + (int64_t)rr * p.lda] : A[rr + (int64_t)kk * p.lda])
                             : (p.tb ? B[rr + (int64_t)kk * p.ldb] : B[kk + (int64_t)rr * p.ldb]);
        const unsigned long long b = (unsigned long long)__double_as_longlong(fabs(v));
        best = b > best ? b : best;
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_down_sync(0xffffffffu, best, off);
        best = o > best ? o : best;
      }
      if (lane == 0) (row ? e_row : f_col)[rr] = exponent_of_max(best);
    }
    __syncthreads();
  }
  for (int m0 = 0; m0 < m; m0 += EM_BM)
    for (int n0 = 0; n0 < n; n0 += EM_BM) {
      if (fp64) {
        emu_tile_fp64(p, m0, n0);
        __syncthreads();
        continue;
      }
      // a tile whose rows or columns hold Inf/NaN: the FP64 loop
      if (tid == 0) s_special = 0;
      __syncthreads();
      if (tid < 2 * EM_BM) {
        const bool row = tid < EM_BM;
        const int r = row ? m0 + tid : n0 + tid - EM_BM;
        if (r < (row ? m : n) && (row ? e_row[r] : f_col[r]) == NONFINITE) s_special = 1;
      }
      __syncthreads();
      if (s_special) {
        emu_tile_fp64(p, m0, n0);
        __syncthreads();
        continue;
      }
      int lev[EM_S][4];
#pragma unroll
      for (int l = 0; l < EM_S; ++l)
#pragma unroll
        for (int c = 0; c < 4; ++c) lev[l][c] = 0;
      for (int k0 = 0; k0 < k; k0 += EM_KC) {
        // digits of the chunk: op(A)(m0 + i, k0 + kk) and op(B)(k0 + kk, n0 + j)
        for (int e = tid; e < EM_BM * EM_KC; e += EM_NT) {
          // A: i fastest when op(A) columns are contiguous (ta = 0), else kk fastest
          const int i = p.ta ? e / EM_KC : e % EM_BM, kk = p.ta ? e % EM_KC : e / EM_BM;
          const int gi = m0 + i, gk = k0 + kk;
          double x = 0.0;
          if (gi < m && gk < k) x = p.ta ? A[gk + (int64_t)gi * p.lda] : A[gi + (int64_t)gk * p.lda];
          bool neg;
          const unsigned long long mag = digit_magnitude(x, gi < m ? e_row[gi] : 0, EM_S, neg);
#pragma unroll
          for (int sl = 0; sl < EM_S; ++sl) {
            const int d = (int)((mag >> (DIGIT_BITS * (EM_S - 1 - sl))) & DIGIT_MASK);
            As[((size_t)sl * EM_BM + i) * EM_KP + kk] = __float2bfloat16_rn((float)(neg ? -d : d));
          }
          // B: kk fastest when op(B) columns are contiguous (tb = 0)
          const int j = p.tb ? e % EM_BM : e / EM_KC, kb = p.tb ? e / EM_BM : e % EM_KC;
          const int gj = n0 + j, gkb = k0 + kb;
          double y = 0.0;
          if (gj < n && gkb < k)
            y = p.tb ? B[gj + (int64_t)gkb * p.ldb] : B[gkb + (int64_t)gj * p.ldb];
          const unsigned long long magb = digit_magnitude(y, gj < n ? f_col[gj] : 0, EM_S, neg);
#pragma unroll
          for (int sl = 0; sl < EM_S; ++sl) {
            const int d = (int)((magb >> (DIGIT_BITS * (EM_S - 1 - sl))) & DIGIT_MASK);
            Bs[((size_t)sl * EM_BM + j) * EM_KP + kb] = __float2bfloat16_rn((float)(neg ? -d : d));
          }
        }
        __syncthreads();
        // the Ozaki triangle: products of level L = s + t <= S + 1 (s, t 1-based)
#pragma unroll
        for (int L = 2; L <= EM_S + 1; ++L) {
          const int s_lo = L - EM_S > 1 ? L - EM_S : 1, s_hi = L - 1 < EM_S ? L - 1 : EM_S;
#pragma unroll 1
          for (int s1 = s_lo; s1 <= s_hi; ++s1) {
            const int t1 = L - s1;
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            const __nv_bfloat16 *as = As + (size_t)(s1 - 1) * EM_BM * EM_KP;
            const __nv_bfloat16 *bs = Bs + (size_t)(t1 - 1) * EM_BM * EM_KP;
#pragma unroll
            for (int ks = 0; ks < EM_KC; ks += 16) {
              uint32_t a[4];
              a[0] = *reinterpret_cast<const uint32_t *>(as + (wm + g) * EM_KP + ks + 2 * tg);
              a[1] = *reinterpret_cast<const uint32_t *>(as + (wm + g + 8) * EM_KP + ks + 2 * tg);
              a[2] = *reinterpret_cast<const uint32_t *>(as + (wm + g) * EM_KP + ks + 2 * tg + 8);
              a[3] = *reinterpret_cast<const uint32_t *>(as + (wm + g + 8) * EM_KP + ks + 2 * tg + 8);
              const __nv_bfloat16 *bc = bs + (wn + g) * EM_KP + ks + 2 * tg;
              mma_bf16_16816(acc, a, *reinterpret_cast<const uint32_t *>(bc),
                             *reinterpret_cast<const uint32_t *>(bc + 8));
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) lev[L - 2][c] += __float2int_rn(acc[c]);
          }
        }
        __syncthreads();  // the slices are rewritten by the next chunk
      }
      // recombine the thread's 4 elements: rows g, g + 8 of the warp's
      // sub-tile, columns 2 tg, 2 tg + 1
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int il = wm + g + (c >= 2 ? 8 : 0), jl = wn + 2 * tg + (c & 1);
          const int i = m0 + il, j = n0 + jl;
          if (i >= m || j >= n) continue;
          __int128 acc = 0;
#pragma unroll
          for (int l = 0; l < EM_S; ++l) acc += (__int128)lev[l][c] << (DIGIT_BITS * (EM_S - 1 - l));
          const double v = level_value(acc, EM_S, e_row[i], f_col[j], p.alpha);
          double *cp = C + i + (int64_t)j * p.ldc;
          *cp = (p.beta == 0.0) ? v : fma(p.beta, *cp, v);
        }
      __syncthreads();
    }
}

__global__ void __launch_bounds__(EM_NT, 2)
grouped_emu_kernel(const DevProblem *__restrict__ probs, const int *__restrict__ order, int count,
                   int *__restrict__ next) {
  extern __shared__ __align__(16) unsigned char emsm[];
  __shared__ int s_idx;
  for (;;) {
    if (threadIdx.x == 0) s_idx = atomicAdd(next, 1);
    __syncthreads();
    const int q = s_idx;
    __syncthreads();
    if (q >= count) break;
    cta_dgemm_emu(probs[order[q]], emsm);
    __syncthreads();
  }
}

// ---------------------------------------------------------------- reductions
template <typename T, int NT>
__device__ void cta_argmax(T val, int idx, T *sv, int *si, T *bv, int *bi) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    T ov = __shfl_down_sync(0xffffffffu, val, off);
    int oi = __shfl_down_sync(0xffffffffu, idx, off);
    if (ov > val || (ov == val && oi < idx)) {
      val = ov;
      idx = oi;
    }
  }
  if (lane == 0) {
    sv[warp] = val;
    si[warp] = idx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    T v = sv[0];
    int i = si[0];
    for (int w = 1; w < NT / 32; ++w)
      if (sv[w] > v || (sv[w] == v && si[w] < i)) {
        v = sv[w];
        i = si[w];
      }
    *bv = v;
    *bi = i;
  }
  __syncthreads();
}

// ---------------------------------------------------------------- LU (one CTA)
// Right-looking LU of an n x n matrix at M (leading dimension ld) with the
// getf2_k.c rules.  ipiv 1-based.  Returns info.
template <typename T, int NT>
__device__ int cta_getrf(int n, T *M, int ld, int *ipiv) {
  __shared__ T sv[NT / 32];
  __shared__ int si[NT / 32];
  __shared__ T s_piv;
  __shared__ int s_p;
  __shared__ T s_rcp;
  const T tiny = sizeof(T) == 8 ? (T)DBL_MIN : (T)FLT_MIN;
  int info = 0;
  for (int j = 0; j < n; ++j) {
    T best = T(-1);
    int bidx = 1 << 30;
    for (int i = j + threadIdx.x; i < n; i += NT) {
      T a = M[i + (int64_t)j * ld];
      a = a < T(0) ? -a : a;
      if (a > best) {  // rows visited in increasing order: first maximum per thread
        best = a;
        bidx = i;
      }
    }
    cta_argmax<T, NT>(best, bidx, sv, si, &s_piv, &s_p);
    const int p = s_p;
    const T piv = M[p + (int64_t)j * ld];
    const T apiv = piv < T(0) ? -piv : piv;
    const bool nonzero = piv != T(0);
    const bool scaled = nonzero && apiv >= tiny;
    // one division per CTA (FP64 divisions are ~10 operations on GB300's
    // scarce FP64 units), shared after the barrier
    if (threadIdx.x == 0) s_rcp = scaled ? T(1) / piv : T(1);
    __syncthreads();  // every thread has the pivot before any row moves
    if (threadIdx.x == 0) ipiv[j] = p + 1;
    if (!nonzero && info == 0) info = j + 1;
    // interchange rows j and p: all columns when scaled, columns > j otherwise
    if (p != j)
      for (int c = threadIdx.x; c < n; c += NT)
        if (scaled || c > j) {
          T t = M[j + (int64_t)c * ld];
          M[j + (int64_t)c * ld] = M[p + (int64_t)c * ld];
          M[p + (int64_t)c * ld] = t;
        }
    __syncthreads();
    if (scaled) {
      const T r = s_rcp;
      for (int i = j + 1 + threadIdx.x; i < n; i += NT) M[i + (int64_t)j * ld] *= r;
    }
    __syncthreads();
    const int rows = n - j - 1;
    const int64_t total = (int64_t)rows * rows;
    for (int64_t e = threadIdx.x; e < total; e += NT) {
      const int i = j + 1 + (int)(e % rows), c = j + 1 + (int)(e / rows);
      M[i + (int64_t)c * ld] = fma(-M[i + (int64_t)j * ld], M[j + (int64_t)c * ld],
                                   M[i + (int64_t)c * ld]);
    }
    __syncthreads();
  }
  return info;
}

// Blocked LU of an n x n matrix at M (leading dimension ld), 16-column
// panels (the structure of lapack/getrf/getrf_single.c): the panel is
// factored in shared memory P (rows x jb, column-major, ld = rows) with the
// getf2_k.c rules, its interchanges are applied to the columns left of the
// panel and to the columns right of it (laswp), and U12 and A22 receive the
// panel's rank-1 updates in column order, each element read and written once
// per panel.  ipiv 1-based.  Returns info.
template <typename T, int NT>
__device__ int cta_getrf_blk(int n, T *M, int ld, int *ipiv, T *P) {
  __shared__ T sv[NT / 32];
  __shared__ int si[NT / 32];
  __shared__ T s_piv;
  __shared__ int s_p;
  __shared__ T s_rcp;
  const T tiny = sizeof(T) == 8 ? (T)DBL_MIN : (T)FLT_MIN;
  int info = 0;
  for (int j0 = 0; j0 < n; j0 += PANEL_B) {
    const int jb = (n - j0) < PANEL_B ? (n - j0) : PANEL_B;
    const int rows = n - j0;
    for (int e = threadIdx.x; e < rows * jb; e += NT) {
      const int r = e % rows, c = e / rows;
      P[e] = M[(j0 + r) + (int64_t)(j0 + c) * ld];
    }
    __syncthreads();
    // ---- panel (getf2) in shared memory
    for (int j = 0; j < jb; ++j) {
      T best = T(-1);
      int bidx = 1 << 30;
      for (int r = j + threadIdx.x; r < rows; r += NT) {
        T a = P[r + j * rows];
        a = a < T(0) ? -a : a;
        if (a > best) {  // rows visited in increasing order: first maximum per thread
          best = a;
          bidx = r;
        }
      }
      cta_argmax<T, NT>(best, bidx, sv, si, &s_piv, &s_p);
      const int p = s_p;
      const T piv = P[p + j * rows];
      const T apiv = piv < T(0) ? -piv : piv;
      const bool nonzero = piv != T(0);
      const bool scaled = nonzero && apiv >= tiny;
      if (threadIdx.x == 0) s_rcp = scaled ? T(1) / piv : T(1);  // one division per CTA
      __syncthreads();  // every thread has the pivot before any row moves
      if (threadIdx.x == 0) ipiv[j0 + j] = j0 + p + 1;
      if (!nonzero && info == 0) info = j0 + j + 1;
      if (p != j)
        for (int c = threadIdx.x; c < jb; c += NT)
          if (scaled || c > j) {
            const T t = P[j + c * rows];
            P[j + c * rows] = P[p + c * rows];
            P[p + c * rows] = t;
          }
      __syncthreads();
      if (scaled) {
        const T r = s_rcp;
        for (int i = j + 1 + threadIdx.x; i < rows; i += NT) P[i + j * rows] *= r;
      }
      __syncthreads();
      const int pr = rows - j - 1, pc = jb - j - 1;
      for (int e = threadIdx.x; e < pr * pc; e += NT) {
        const int i = j + 1 + e % pr, c = j + 1 + e / pr;
        P[i + c * rows] = fma(-P[i + j * rows], P[j + c * rows], P[i + c * rows]);
      }
      __syncthreads();
    }
    for (int e = threadIdx.x; e < rows * jb; e += NT) {
      const int r = e % rows, c = e / rows;
      M[(j0 + r) + (int64_t)(j0 + c) * ld] = P[e];
    }
    // ---- the panel's interchanges on the other columns (one thread per column)
    for (int c = threadIdx.x; c < n; c += NT) {
      if (c >= j0 && c < j0 + jb) continue;
      T *col = M + (int64_t)c * ld;
      for (int j = 0; j < jb; ++j) {
        const int p = ipiv[j0 + j] - 1;
        if (p != j0 + j) {
          const T t = col[j0 + j];
          col[j0 + j] = col[p];
          col[p] = t;
        }
      }
    }
    __syncthreads();
    const int ncols = n - j0 - jb;
    if (ncols <= 0) continue;
    // ---- U12: row t of the right columns takes the multipliers of rows < t
    for (int c = threadIdx.x; c < ncols; c += NT) {
      T *col = M + (int64_t)(j0 + jb + c) * ld + j0;
      for (int t = 1; t < jb; ++t) {
        T a = col[t];
        for (int k = 0; k < t; ++k) a = fma(-P[t + k * rows], col[k], a);
        col[t] = a;
      }
    }
    __syncthreads();
    // ---- A22 -= L21 U12, k in column order
    const int mr = rows - jb;
    const int64_t total = (int64_t)mr * ncols;
    for (int64_t e = threadIdx.x; e < total; e += NT) {
      const int i = (int)(e % mr), c = (int)(e / mr);
      const T *u = M + (int64_t)(j0 + jb + c) * ld + j0;
      T *dst = M + (j0 + jb + i) + (int64_t)(j0 + jb + c) * ld;
      T a = *dst;
#pragma unroll 4
      for (int k = 0; k < jb; ++k) a = fma(-P[(jb + i) + k * rows], u[k], a);
      *dst = a;
    }
    __syncthreads();
  }
  return info;
}

// Solve (LU) X = P B for nrhs columns (B overwritten), forward/back
// substitution.  Each right-hand side is staged in shared memory `w` (n
// entries): the interchanges, applied in order by one thread, and the two
// triangular sweeps then touch shared memory only.
template <typename TM, typename TB_, int NT>
__device__ void cta_getrs(int n, int nrhs, const TM *LU, int ld, const int *ipiv, TB_ *B,
                          int ldb, TB_ *w) {
  for (int r = 0; r < nrhs; ++r) {
    TB_ *b = B + (int64_t)r * ldb;
    for (int i = threadIdx.x; i < n; i += NT) w[i] = b[i];
    __syncthreads();
    if (threadIdx.x == 0)
      for (int i = 0; i < n; ++i) {
        const int p = ipiv[i] - 1;
        if (p != i) {
          TB_ t = w[i];
          w[i] = w[p];
          w[p] = t;
        }
      }
    __syncthreads();
    for (int j = 0; j < n; ++j) {  // L y = b (unit diagonal)
      const TB_ xj = w[j];
      for (int i = j + 1 + threadIdx.x; i < n; i += NT)
        w[i] = fma(-(TB_)LU[i + (int64_t)j * ld], xj, w[i]);
      __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {  // U x = y
      if (threadIdx.x == 0) w[j] = w[j] / (TB_)LU[j + (int64_t)j * ld];
      __syncthreads();
      const TB_ xj = w[j];
      for (int i = threadIdx.x; i < j; i += NT) w[i] = fma(-(TB_)LU[i + (int64_t)j * ld], xj, w[i]);
      __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += NT) b[i] = w[i];
    __syncthreads();
  }
}

// ---------------------------------------------------------------- POTRF
template <int NT>
__device__ int cta_potrf(int n, double *M, int ld, bool upper) {
  __shared__ double s_d, s_r;
  __shared__ int s_fail;
  auto at = [&](int i, int c) -> double & {  // element (i, c) of the lower view
    return upper ? M[c + (int64_t)i * ld] : M[i + (int64_t)c * ld];
  };
  for (int j = 0; j < n; ++j) {
    if (threadIdx.x == 0) {
      const double ajj = at(j, j);
      s_fail = 0;
      if (ajj <= 0.0) {
        s_fail = 1;  // potf2_L.c:67-71: write the pivot back, info = j + 1
      } else {
        at(j, j) = sqrt(ajj);
      }
      s_d = at(j, j);
      s_r = 1.0 / s_d;  // one division per CTA
    }
    __syncthreads();
    if (s_fail) return j + 1;
    const double r = s_r;
    for (int i = j + 1 + threadIdx.x; i < n; i += NT) at(i, j) *= r;
    __syncthreads();
    const int rows = n - j - 1;
    const int64_t total = (int64_t)rows * rows;
    for (int64_t e = threadIdx.x; e < total; e += NT) {
      const int i = j + 1 + (int)(e % rows), c = j + 1 + (int)(e / rows);
      if (i >= c) at(i, c) = fma(-at(i, j), at(c, j), at(i, c));
    }
    __syncthreads();
  }
  return 0;
}

// Blocked Cholesky (16-column panels in shared memory P, rows x jb): the
// operations of cta_potrf per element and in the same order.  On a
// non-positive pivot the columns before it are final and everything after it
// carries exactly the updates of those columns, as in the unblocked form.
template <int NT>
__device__ int cta_potrf_blk(int n, double *M, int ld, bool upper, double *P) {
  __shared__ double s_d, s_r;
  __shared__ int s_fail;
  auto at = [&](int i, int c) -> double & {  // element (i, c) of the lower view
    return upper ? M[c + (int64_t)i * ld] : M[i + (int64_t)c * ld];
  };
  for (int j0 = 0; j0 < n; j0 += PANEL_B) {
    const int jb = (n - j0) < PANEL_B ? (n - j0) : PANEL_B;
    const int rows = n - j0;
    for (int e = threadIdx.x; e < rows * jb; e += NT) {
      const int r = e % rows, c = e / rows;
      if (r >= c) P[e] = at(j0 + r, j0 + c);
    }
    __syncthreads();
    int done = jb;  // panel columns completed
    for (int j = 0; j < jb; ++j) {
      if (threadIdx.x == 0) {
        const double ajj = P[j + j * rows];
        s_fail = 0;
        if (ajj <= 0.0) s_fail = 1;  // potf2_L.c:67-71: the pivot stays, info = j + 1
        else P[j + j * rows] = sqrt(ajj);
        s_d = P[j + j * rows];
        s_r = 1.0 / s_d;  // one division per CTA
      }
      __syncthreads();
      if (s_fail) {
        done = j;
        break;
      }
      const double r = s_r;
      for (int i = j + 1 + threadIdx.x; i < rows; i += NT) P[i + j * rows] *= r;
      __syncthreads();
      const int pr = rows - j - 1, pc = jb - j - 1;
      for (int e = threadIdx.x; e < pr * pc; e += NT) {
        const int i = j + 1 + e % pr, c = j + 1 + e / pr;
        if (i >= c) P[i + c * rows] = fma(-P[i + j * rows], P[c + j * rows], P[i + c * rows]);
      }
      __syncthreads();
    }
    for (int e = threadIdx.x; e < rows * jb; e += NT) {
      const int r = e % rows, c = e / rows;
      if (r >= c) at(j0 + r, j0 + c) = P[e];
    }
    // trailing lower triangle: the updates of the completed panel columns
    const int mr = rows - jb;
    const int64_t total = (int64_t)mr * mr;
    for (int64_t e = threadIdx.x; e < total; e += NT) {
      const int i = (int)(e % mr), c = (int)(e / mr);
      if (i < c) continue;
      double a = at(j0 + jb + i, j0 + jb + c);
      for (int k = 0; k < done; ++k)
        a = fma(-P[(jb + i) + k * rows], P[(jb + c) + k * rows], a);
      at(j0 + jb + i, j0 + jb + c) = a;
    }
    __syncthreads();
    if (done < jb) return j0 + done + 1;
  }
  return 0;
}

// ---------------------------------------------------------------- mixed DGESV
template <int NT>
__device__ int cta_dsgesv(const DevProblem &p, double *smem, int blk_nmax) {
  const int n = p.n, nrhs = p.k;
  double *A = (double *)p.A;
  double *B = (double *)p.B;
  int *ipiv = (int *)p.C;
  float *S = p.work;            // n x n FP32 factors
  float *sr = S + (int64_t)n * n;  // FP32 correction (n)
  double *x = (double *)(sr + n);  // FP64 iterate (n); n*n + n floats keep 8-byte alignment
  __shared__ double red[NT / 32];
  __shared__ int s_ok;
  __shared__ double s_anrm;
  // ||A||_inf and the FP32 copy of A
  {
    double best = 0.0;
    for (int i = threadIdx.x; i < n; i += NT) {
      double s = 0.0;
      for (int c = 0; c < n; ++c) s += fabs(A[i + (int64_t)c * p.lda]);
      best = s > best ? s : best;
    }
    for (int off = 16; off > 0; off >>= 1) best = fmax(best, __shfl_down_sync(0xffffffffu, best, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = 0.0;
      for (int w = 0; w < NT / 32; ++w) b = fmax(b, red[w]);
      s_anrm = b;
    }
    for (int64_t e = threadIdx.x; e < (int64_t)n * n; e += NT) {
      const int i = (int)(e % n), c = (int)(e / n);
      S[e] = (float)A[i + (int64_t)c * p.lda];
    }
    __syncthreads();
  }
  const double cte = s_anrm * (DBL_EPSILON * 0.5) * sqrt((double)n);
  int sinfo = n <= blk_nmax ? cta_getrf_blk<float, NT>(n, S, n, ipiv, reinterpret_cast<float *>(smem))
                            : cta_getrf<float, NT>(n, S, n, ipiv);
  __syncthreads();
  bool ok = sinfo == 0;
  int r = 0;  // columns < r hold converged solutions
  for (; r < nrhs && ok; ++r) {
    double *b = B + (int64_t)r * p.ldb;
    // x0 = fp64(LU32 \ fp32(b))
    for (int i = threadIdx.x; i < n; i += NT) sr[i] = (float)b[i];
    __syncthreads();
    cta_getrs<float, float, NT>(n, 1, S, n, ipiv, sr, n, reinterpret_cast<float *>(smem));
    for (int i = threadIdx.x; i < n; i += NT) x[i] = (double)sr[i];
    __syncthreads();
    bool conv = false;
    for (int it = 0; it <= 30; ++it) {
      // r = b - A x (FP64), max|r| and max|x|
      double rmax = 0.0, xmax = 0.0;
      for (int i = threadIdx.x; i < n; i += NT) {
        double s = b[i];
        for (int c = 0; c < n; ++c) s = fma(-A[i + (int64_t)c * p.lda], x[c], s);
        sr[i] = (float)s;
        rmax = fmax(rmax, fabs(s));
        xmax = fmax(xmax, fabs(x[i]));
      }
      for (int off = 16; off > 0; off >>= 1) {
        rmax = fmax(rmax, __shfl_down_sync(0xffffffffu, rmax, off));
        xmax = fmax(xmax, __shfl_down_sync(0xffffffffu, xmax, off));
      }
      __syncthreads();
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = rmax;
      __syncthreads();
      if (threadIdx.x == 0) {
        double b2 = 0.0;
        for (int w = 0; w < NT / 32; ++w) b2 = fmax(b2, red[w]);
        s_anrm = b2;  // reuse as max|r|
      }
      __syncthreads();
      const double rm = s_anrm;
      __syncthreads();
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = xmax;
      __syncthreads();
      if (threadIdx.x == 0) {
        double b2 = 0.0;
        for (int w = 0; w < NT / 32; ++w) b2 = fmax(b2, red[w]);
        s_ok = rm <= b2 * cte;
      }
      __syncthreads();
      if (s_ok) {
        conv = true;
        break;
      }
      cta_getrs<float, float, NT>(n, 1, S, n, ipiv, sr, n, reinterpret_cast<float *>(smem));
      for (int i = threadIdx.x; i < n; i += NT) x[i] += (double)sr[i];
      __syncthreads();
    }
    if (!conv) {
      ok = false;
      break;
    }
    for (int i = threadIdx.x; i < n; i += NT) b[i] = x[i];
    __syncthreads();
  }
  if (ok) return 0;
  // FP64 fallback (dsgesv.f:410-425): factor A in place and solve the
  // right-hand sides that have no converged solution yet
  const int info = n <= blk_nmax ? cta_getrf_blk<double, NT>(n, A, p.lda, ipiv, smem)
                                 : cta_getrf<double, NT>(n, A, p.lda, ipiv);
  __syncthreads();
  if (info == 0)
    cta_getrs<double, double, NT>(n, nrhs - r, A, p.lda, ipiv, B + (int64_t)r * p.ldb, p.ldb,
                                  smem);
  return info;
}

// ---------------------------------------------------------------- kernel
// Dynamic shared memory of the grouped kernel: the DGEMM tiles, or the
// panel of the blocked LU / Cholesky (blk_nmax rows x PANEL_B columns).
constexpr int BLK_SMEM_MAX = 96 * 1024;
// Largest LU / Cholesky order of a batched problem.  A right-hand side is
// staged in the kernel's shared memory, which holds PANEL_B doubles per row
// of the largest order factored by panels, and BLK_SMEM_MAX / 8 = 12288
// doubles once that order is capped.
constexpr int BATCH_MAX_ORDER = BLK_SMEM_MAX / (int)sizeof(double);
__host__ __device__ constexpr size_t grouped_smem(int blk_nmax) {
  return (size_t)blk_nmax * PANEL_B * sizeof(double) > 2 * DG_BK * 64 * sizeof(double)
             ? (size_t)blk_nmax * PANEL_B * sizeof(double)
             : 2 * DG_BK * 64 * sizeof(double);
}

template <int NT>
__global__ void __launch_bounds__(NT)
grouped_kernel(const DevProblem *__restrict__ probs, const int *__restrict__ order, int count,
               int *__restrict__ next, int mixed, int blk_nmax) {
  extern __shared__ __align__(16) double dsm[];
  __shared__ int s_idx;
  for (;;) {
    if (threadIdx.x == 0) s_idx = atomicAdd(next, 1);
    __syncthreads();
    const int q = s_idx;
    __syncthreads();
    if (q >= count) break;
    const DevProblem p = probs[order[q]];
    if (p.type == GB_BATCH_DGEMM) {
      if (p.tile == 32)
        cta_dgemm<NT, 32>(p, dsm);
      else
        cta_dgemm<NT, 64>(p, dsm);
    } else if (p.type == GB_BATCH_DGESV) {
      int info;
      if (mixed) {
        info = cta_dsgesv<NT>(p, dsm, blk_nmax);
      } else {
        info = p.n <= blk_nmax
                   ? cta_getrf_blk<double, NT>(p.n, (double *)p.A, p.lda, (int *)p.C, dsm)
                   : cta_getrf<double, NT>(p.n, (double *)p.A, p.lda, (int *)p.C);
        __syncthreads();
        if (info == 0)
          cta_getrs<double, double, NT>(p.n, p.k, (const double *)p.A, p.lda, (const int *)p.C,
                                        (double *)p.B, p.ldb, dsm);
      }
      if (threadIdx.x == 0 && p.info) *p.info = info;
    } else if (p.type == GB_BATCH_DPOTRF) {
      const int info = p.n <= blk_nmax
                           ? cta_potrf_blk<NT>(p.n, (double *)p.A, p.lda, p.uplo == 0, dsm)
                           : cta_potrf<NT>(p.n, (double *)p.A, p.lda, p.uplo == 0);
      if (threadIdx.x == 0 && p.info) *p.info = info;
    }
    __syncthreads();
  }
}

double problem_cost(const gb_batch_problem &p) {
  const double n = p.n, m = p.m, k = p.k;
  if (p.type == GB_BATCH_DGEMM) return 2.0 * m * n * k;
  if (p.type == GB_BATCH_DGESV) return 2.0 / 3.0 * n * n * n + 2.0 * n * n * k;
  return n * n * n / 3.0;
}

}  // namespace

// ------------------------------------------------------------------ plan
struct BatchPlan {
  std::string key;
  int count = 0;
  int mixed = 0;
  int threads = 256;
  DevProblem *d_probs = nullptr;
  int *d_order = nullptr;
  int *d_next = nullptr;
  int *d_loopnext = nullptr;
  float *d_work = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int emulated = 0;      // DGEMM problems on the emulated-FP64 kernel
  int *d_order_emu = nullptr;  // their order (the other problems stay in d_order)
  int count_emu = 0, count_main = 0;
  std::vector<int> h_order, h_order_emu;  // host copies of both orders
  int blk_nmax = 0;      // LU/Cholesky problems up to this order use the blocked forms
  size_t smem = 0;       // dynamic shared memory of the grouped kernel
  std::vector<int> bin_tile;  // DGEMM tile edge per size bin (autotuned)
  std::vector<DevProblem> host_probs;  // the table as uploaded (tiles re-set by the tuner)
};

namespace {

// What the autotuner found for a histogram key: threads per CTA and the
// DGEMM tile edge of every size bin.
struct Tuned {
  int threads = 0;
  int tile[TILE_BINS] = {0, 0, 0, 0};
};
std::mutex g_tune_mu;
std::map<std::string, Tuned> g_tuned;  // histogram key -> tuned choice

// The grouped kernel's instances accept up to BLK_SMEM_MAX bytes of dynamic
// shared memory (set once per device).
int grouped_smem_attr() {
  static PerDeviceOnce once;
  return once.run(current_device(), [] {
    GB_CUDA(cudaFuncSetAttribute(grouped_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 BLK_SMEM_MAX));
    GB_CUDA(cudaFuncSetAttribute(grouped_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 BLK_SMEM_MAX));
    GB_CUDA(cudaFuncSetAttribute(grouped_kernel<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 BLK_SMEM_MAX));
    return GB_SUCCESS;
  });
}

// CTAs of the persistent grouped kernel: as many as fit on every SM (a CTA
// waiting at a barrier of a small problem leaves the FP64 pipe to the others).
int grouped_grid(int threads, size_t smem) {
  int per_sm = 0;
  cudaError_t e = cudaErrorInvalidValue;
  if (threads == 128)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grouped_kernel<128>, 128, smem);
  else if (threads == 512)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grouped_kernel<512>, 512, smem);
  else
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grouped_kernel<256>, 256, smem);
  if (e != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 2;
  }
  if (per_sm > 8) per_sm = 8;
  return sm_count() * per_sm;
}

// One launch of the grouped kernel over `count` entries of `order`.
int launch_grouped_on(BatchPlan *pl, int threads, const int *order, int count, int *next,
                      int grid, cudaStream_t s) {
  int st = grouped_smem_attr();
  if (st) return st;
  if (grid <= 0) grid = grouped_grid(threads, pl->smem);
  GB_CUDA(cudaMemsetAsync(next, 0, sizeof(int), s));
  const size_t sm = pl->smem;
  if (threads == 128)
    grouped_kernel<128><<<grid, 128, sm, s>>>(pl->d_probs, order, count, next, pl->mixed,
                                              pl->blk_nmax);
  else if (threads == 512)
    grouped_kernel<512><<<grid, 512, sm, s>>>(pl->d_probs, order, count, next, pl->mixed,
                                              pl->blk_nmax);
  else
    grouped_kernel<256><<<grid, 256, sm, s>>>(pl->d_probs, order, count, next, pl->mixed,
                                              pl->blk_nmax);
  count_launch();
  return check_cuda(cudaGetLastError(), "grouped batch launch");
}

int emu_attr() {
  static PerDeviceOnce once;
  return once.run(current_device(), [] {
    GB_CUDA(cudaFuncSetAttribute(grouped_emu_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)EM_SMEM));
    return GB_SUCCESS;
  });
}

int launch_grouped_emu(BatchPlan *pl, const int *order, int count, int *next, cudaStream_t s) {
  int st = emu_attr();
  if (st) return st;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grouped_emu_kernel, EM_NT, EM_SMEM) !=
          cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  GB_CUDA(cudaMemsetAsync(next, 0, sizeof(int), s));
  grouped_emu_kernel<<<sm_count() * per_sm, EM_NT, EM_SMEM, s>>>(pl->d_probs, order, count, next);
  count_launch();
  return check_cuda(cudaGetLastError(), "grouped emulated batch launch");
}

int launch_grouped(BatchPlan *pl, int threads, cudaStream_t s);

// The plan's launches captured in a CUDA graph (pl->graph / pl->exec).  With
// both kernels (emulated DGEMM problems and the rest) the graph forks: the two
// persistent kernels run side by side and join at the end.
void capture_plan(BatchPlan *pl) {
  cudaStream_t cap = nullptr, cap2 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  const bool both = pl->count_emu > 0 && pl->count_main > 0;
  if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  bool ok = !both || (cudaStreamCreateWithFlags(&cap2, cudaStreamNonBlocking) == cudaSuccess &&
                      cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) == cudaSuccess &&
                      cudaEventCreateWithFlags(&join, cudaEventDisableTiming) == cudaSuccess);
  if (ok && cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    int st = GB_SUCCESS;
    if (both) {
      cudaEventRecord(fork, cap);
      cudaStreamWaitEvent(cap2, fork, 0);
      st = launch_grouped_emu(pl, pl->d_order_emu, pl->count_emu, pl->d_next + 1, cap2);
      if (!st) st = launch_grouped_on(pl, pl->threads, pl->d_order, pl->count_main, pl->d_next, 0,
                                      cap);
      cudaEventRecord(join, cap2);
      cudaStreamWaitEvent(cap, join, 0);
    } else {
      st = launch_grouped(pl, pl->threads, cap);
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamEndCapture(cap, &g) == cudaSuccess && !st &&
        cudaGraphInstantiate(&pl->exec, g, 0) == cudaSuccess) {
      pl->graph = g;
    } else {
      if (g) cudaGraphDestroy(g);
      pl->exec = nullptr;
    }
  }
  cudaGetLastError();
  if (fork) cudaEventDestroy(fork);
  if (join) cudaEventDestroy(join);
  if (cap2) cudaStreamDestroy(cap2);
  cudaStreamDestroy(cap);
}

int launch_grouped(BatchPlan *pl, int threads, cudaStream_t s) {
  int st = GB_SUCCESS;
  if (pl->count_emu > 0 &&
      (st = launch_grouped_emu(pl, pl->d_order_emu, pl->count_emu, pl->d_next + 1, s)))
    return st;
  if (pl->count_main > 0)
    st = launch_grouped_on(pl, threads, pl->d_order, pl->count_main, pl->d_next, 0, s);
  return st;
}

// Size bins of the DGEMM tile choice: the larger of m and n.
inline int tile_bin(int m, int n) {
  const int d = m > n ? m : n;
  return d <= 48 ? 0 : d <= 96 ? 1 : d <= 160 ? 2 : 3;
}
// Untuned default: 32x32 tiles up to 96 (less padding), 64x64 above.
inline int default_tile(int bin) { return bin <= 1 ? 32 : 64; }

// Key of the autotuner: type counts and a log2 histogram of the dominant size.
std::string histogram_key(const std::vector<gb_batch_problem> &v, int mixed) {
  int hist[3][10] = {{0}};
  for (const auto &p : v) {
    const int sz = p.type == GB_BATCH_DGEMM ? std::max(p.m, std::max(p.n, p.k)) : p.n;
    int b = 0;
    while (b < 9 && (1 << (b + 3)) < sz) ++b;
    const int t = p.type < 0 ? 0 : (p.type > 2 ? 2 : p.type);
    hist[t][b]++;
  }
  std::string key = "fp64:" + std::to_string(mixed) + ":";
  for (int t = 0; t < 3; ++t)
    for (int b = 0; b < 10; ++b) {
      // coarse (log2) counts keep similar batches on the same entry
      int c = hist[t][b], lg = 0;
      while (c > 0) {
        c >>= 1;
        ++lg;
      }
      key += std::to_string(lg) + ",";
    }
  return key;
}

}  // namespace

}  // namespace gb

using namespace gb;

extern "C" {

void *gb_batch_plan_create(const gb_batch_problem *problems, int count, int flags) {
  if (count < 0 || (count > 0 && !problems)) {
    set_error(GB_ERR_INVALID_VALUE, "gb_batch_plan_create: bad problem list");
    return nullptr;
  }
  for (int i = 0; i < count; ++i) {
    const gb_batch_problem &p = problems[i];
    const bool bad = p.type < GB_BATCH_DGEMM || p.type > GB_BATCH_DPOTRF || p.n < 0 ||
                     (p.type == GB_BATCH_DGEMM && (p.m < 0 || p.k < 0 || p.ldc < (p.m > 1 ? p.m : 1))) ||
                     (p.type != GB_BATCH_DGEMM && p.lda < (p.n > 1 ? p.n : 1)) ||
                     (p.type == GB_BATCH_DGESV && (p.k < 0 || p.ldb < (p.n > 1 ? p.n : 1))) ||
                     (p.type != GB_BATCH_DGEMM && p.n > BATCH_MAX_ORDER);
    if (bad) {
      set_error(GB_ERR_INVALID_VALUE, "gb_batch_plan_create: problem %d is invalid", i);
      return nullptr;
    }
  }
  if (ensure_init()) return nullptr;
  cudaStream_t s = stream();
  BatchPlan *pl = new BatchPlan();
  pl->count = count;
  pl->mixed = (flags & GB_BATCH_MIXED) ? 1 : 0;
  pl->stream = s;
  std::vector<gb_batch_problem> v(problems, problems + count);
  // FP32 scratch for the mixed DGESV variant
  size_t work_floats = 0;
  std::vector<size_t> work_off(count, 0);
  if (pl->mixed)
    for (int i = 0; i < count; ++i)
      if (v[i].type == GB_BATCH_DGESV) {
        work_off[i] = work_floats;
        const size_t nn = (size_t)v[i].n;
        work_floats += nn * nn + 4 * nn + 8;  // factors, correction, FP64 iterate (2 words/entry)
        work_floats = (work_floats + 63) & ~size_t(63);
      }
  std::vector<DevProblem> d(count);
  int nmax = 0;  // largest LU / Cholesky order
  for (int i = 0; i < count; ++i) {
    const gb_batch_problem &p = v[i];
    DevProblem &q = d[i];
    memset(&q, 0, sizeof(q));
    if (p.type != GB_BATCH_DGEMM && p.n > nmax) nmax = p.n;
    q.type = p.type;
    q.m = p.m;
    q.n = p.n;
    q.k = p.k;
    q.ta = (upch(p.transa) == 'T' || upch(p.transa) == 'C') ? 1 : 0;
    q.tb = (upch(p.transb) == 'T' || upch(p.transb) == 'C') ? 1 : 0;
    q.uplo = upch(p.uplo) == 'U' ? 0 : 1;
    q.alpha = p.alpha;
    q.beta = p.beta;
    q.A = p.A;
    q.B = p.B;
    q.C = p.C;
    q.lda = p.lda;
    q.ldb = p.ldb;
    q.ldc = p.ldc;
    q.info = p.info;
  }
  // order: decreasing cost (longest-processing-time first); with the
  // emulated flag the DGEMM problems form their own list for their kernel
  pl->emulated = (flags & GB_BATCH_EMULATED) ? 1 : 0;
  std::vector<int> order, order_emu;
  for (int i = 0; i < count; ++i)
    (pl->emulated && v[i].type == GB_BATCH_DGEMM ? order_emu : order).push_back(i);
  auto lpt = [&](std::vector<int> &o) {
    std::stable_sort(o.begin(), o.end(), [&](int a, int b) {
      return problem_cost(v[a]) > problem_cost(v[b]);
    });
  };
  lpt(order);
  lpt(order_emu);
  pl->count_main = (int)order.size();
  pl->count_emu = (int)order_emu.size();
  pl->h_order = order;
  pl->h_order_emu = order_emu;
  const size_t bytes = sizeof(DevProblem) * (size_t)(count > 0 ? count : 1);
  if (cudaMalloc(&pl->d_probs, bytes) != cudaSuccess ||
      cudaMalloc(&pl->d_order, sizeof(int) * (size_t)(count > 0 ? count : 1)) != cudaSuccess ||
      cudaMalloc(&pl->d_order_emu, sizeof(int) * (size_t)(count > 0 ? count : 1)) != cudaSuccess ||
      cudaMalloc(&pl->d_next, sizeof(int) * 4) != cudaSuccess ||
      (work_floats && cudaMalloc(&pl->d_work, work_floats * sizeof(float)) != cudaSuccess)) {
    check_cuda(cudaErrorMemoryAllocation, "gb_batch_plan_create");
    gb_batch_plan_destroy(pl);
    return nullptr;
  }
  for (int i = 0; i < count; ++i)
    if (pl->mixed && v[i].type == GB_BATCH_DGESV) d[i].work = pl->d_work + work_off[i];
  // blocked LU / Cholesky for the orders whose panel fits the shared memory
  pl->blk_nmax = nmax;
  if ((size_t)pl->blk_nmax * PANEL_B * sizeof(double) > (size_t)BLK_SMEM_MAX)
    pl->blk_nmax = BLK_SMEM_MAX / (PANEL_B * (int)sizeof(double));
  pl->smem = grouped_smem(pl->blk_nmax);
  // DGEMM tiles and CTA size from the autotuner cache (keyed by the
  // problem-size histogram), else the defaults
  const std::string key = histogram_key(v, pl->mixed);
  pl->key = key;
  Tuned tuned;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) tuned = it->second;
  }
  pl->bin_tile.resize(TILE_BINS);
  for (int b = 0; b < TILE_BINS; ++b) pl->bin_tile[b] = tuned.tile[b] ? tuned.tile[b] : default_tile(b);
  for (int i = 0; i < count; ++i)
    if (d[i].type == GB_BATCH_DGEMM) d[i].tile = pl->bin_tile[tile_bin(d[i].m, d[i].n)];
  pl->host_probs = d;
  if (count) {
    cudaError_t e = cudaMemcpy(pl->d_probs, d.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !order.empty())
      e = cudaMemcpy(pl->d_order, order.data(), sizeof(int) * order.size(),
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !order_emu.empty())
      e = cudaMemcpy(pl->d_order_emu, order_emu.data(), sizeof(int) * order_emu.size(),
                     cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      check_cuda(e, "gb_batch_plan_create: table upload");
      gb_batch_plan_destroy(pl);
      return nullptr;
    }
  }
  // untuned default 256 threads; gb_batch_plan_tune refines and caches
  pl->threads = tuned.threads ? tuned.threads : 256;
  // capture the launch(es) in a CUDA graph on private capture streams
  capture_plan(pl);
  return pl;
}

int gb_batch_plan_tune(void *plan) {
  BatchPlan *pl = reinterpret_cast<BatchPlan *>(plan);
  if (!pl) return set_error(GB_ERR_INVALID_VALUE, "gb_batch_plan_tune: null plan");
  if (pl->count == 0) return GB_SUCCESS;
  int st = ensure_init();
  if (st) return st;
  cudaStream_t s = stream();
  cudaEvent_t e0, e1;
  if ((st = check_cuda(cudaEventCreate(&e0), "gb_batch_plan_tune: event"))) return st;
  if ((st = check_cuda(cudaEventCreate(&e1), "gb_batch_plan_tune: event"))) {
    cudaEventDestroy(e0);
    return st;
  }
  auto timed = [&](int threads, const int *order, int cnt, float *ms) -> int {
    cudaEventRecord(e0, s);
    int r = launch_grouped_on(pl, threads, order, cnt, pl->d_next, 0, s);
    if (r) return r;
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    *ms = 0.f;
    cudaEventElapsedTime(ms, e0, e1);
    return GB_SUCCESS;
  };
  auto upload = [&]() -> int {
    return check_cuda(cudaMemcpyAsync(pl->d_probs, pl->host_probs.data(),
                                      sizeof(DevProblem) * pl->host_probs.size(),
                                      cudaMemcpyHostToDevice, s),
                      "gb_batch_plan_tune: table");
  };
  // 1. DGEMM tile edge per size bin: time each candidate on that bin's
  //    problems alone (the same CTA size for both)
  int *d_sub = nullptr;
  st = check_cuda(cudaMalloc(&d_sub, sizeof(int) * (size_t)pl->count), "gb_batch_plan_tune");
  for (int b = 0; b < TILE_BINS && !st; ++b) {
    std::vector<int> sub;
    for (int i = 0; i < pl->count; ++i) {
      const DevProblem &q = pl->host_probs[i];
        if (!pl->emulated && q.type == GB_BATCH_DGEMM && tile_bin(q.m, q.n) == b) sub.push_back(i);
    }
    if (sub.size() < 8) continue;  // too few problems to time
    st = check_cuda(cudaMemcpyAsync(d_sub, sub.data(), sizeof(int) * sub.size(),
                                    cudaMemcpyHostToDevice, s), "gb_batch_plan_tune");
    float best = 1e30f;
    for (int tile : {32, 64}) {
      for (int i : sub) pl->host_probs[i].tile = tile;
      if (st || (st = upload())) break;
      float ms = 0.f;
      if ((st = timed(pl->threads, d_sub, (int)sub.size(), &ms))) break;
      if (ms < best) {
        best = ms;
        pl->bin_tile[b] = tile;
      }
    }
    for (int i : sub) pl->host_probs[i].tile = pl->bin_tile[b];
  }
  cudaFree(d_sub);
  if (!st) st = upload();
  // 2. CTA size on the whole batch with the chosen tiles
  const int cands[3] = {128, 256, 512};
  float best_ms = 1e30f;
  int best_t = pl->threads;
  for (int t : cands) {
    if (st || pl->count_main == 0) break;
    float ms = 0.f;
    if ((st = timed(t, pl->d_order, pl->count_main, &ms))) break;
    if (ms < best_ms) {
      best_ms = ms;
      best_t = t;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  pl->threads = best_t;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    Tuned t;
    t.threads = best_t;
    for (int b = 0; b < TILE_BINS; ++b) t.tile[b] = pl->bin_tile[b];
    g_tuned[pl->key] = t;
  }
  if (config().verbose)
    fprintf(stderr, "libgbblas batch tune: %d threads, DGEMM tiles %d/%d/%d/%d by size bin\n",
            best_t, pl->bin_tile[0], pl->bin_tile[1], pl->bin_tile[2], pl->bin_tile[3]);
  if (pl->exec) {
    cudaGraphExecDestroy(pl->exec);
    pl->exec = nullptr;
  }
  if (pl->graph) {
    cudaGraphDestroy(pl->graph);
    pl->graph = nullptr;
  }
  capture_plan(pl);
  return finish_blocking(s);
}

int gb_batch_plan_threads(void *plan) {
  BatchPlan *pl = reinterpret_cast<BatchPlan *>(plan);
  return pl ? pl->threads : 0;
}

int gb_batch_execute(void *plan) {
  BatchPlan *pl = reinterpret_cast<BatchPlan *>(plan);
  if (!pl) return set_error(GB_ERR_INVALID_VALUE, "gb_batch_execute: null plan");
  int st = ensure_init();
  if (st) return st;
  if (pl->count == 0) return GB_SUCCESS;
  cudaStream_t s = stream();
  if (pl->exec) {
    count_launch();
    return check_cuda(cudaGraphLaunch(pl->exec, s), "cudaGraphLaunch(batch)");
  }
  return launch_grouped(pl, pl->threads, s);
}

int gb_batch_execute_loop(void *plan) {
  BatchPlan *pl = reinterpret_cast<BatchPlan *>(plan);
  if (!pl) return set_error(GB_ERR_INVALID_VALUE, "gb_batch_execute_loop: null plan");
  int st = ensure_init();
  if (st) return st;
  if (pl->count == 0) return GB_SUCCESS;
  cudaStream_t s = stream();
  if (!pl->d_loopnext) {
    if (cudaMalloc(&pl->d_loopnext, sizeof(int) * (size_t)pl->count) != cudaSuccess)
      return check_cuda(cudaErrorMemoryAllocation, "gb_batch_execute_loop");
  }
  GB_CUDA(cudaMemsetAsync(pl->d_loopnext, 0, sizeof(int) * (size_t)pl->count, s));
  // one launch of the same per-problem code for every problem, in table order
  if ((st = grouped_smem_attr())) return st;
  if (pl->count_emu && (st = emu_attr())) return st;
  for (int q = 0; q < pl->count_emu; ++q) {
    grouped_emu_kernel<<<1, EM_NT, EM_SMEM, s>>>(pl->d_probs, pl->d_order_emu + q, 1,
                                                 pl->d_loopnext + q);
    count_launch();
  }
  int *next = pl->d_loopnext + pl->count_emu;
  for (int q = 0; q < pl->count_main; ++q) {
    if (pl->threads == 128)
      grouped_kernel<128><<<1, 128, pl->smem, s>>>(pl->d_probs, pl->d_order + q, 1, next + q,
                                                   pl->mixed, pl->blk_nmax);
    else if (pl->threads == 512)
      grouped_kernel<512><<<1, 512, pl->smem, s>>>(pl->d_probs, pl->d_order + q, 1, next + q,
                                                   pl->mixed, pl->blk_nmax);
    else
      grouped_kernel<256><<<1, 256, pl->smem, s>>>(pl->d_probs, pl->d_order + q, 1, next + q,
                                                   pl->mixed, pl->blk_nmax);
    count_launch();
  }
  return check_cuda(cudaGetLastError(), "batch loop");
}

}  // extern "C"

namespace gb {

// cblas_dgemm_batch after argument checks: all problems go to one grouped
// launch.  Host operands are packed into one pinned buffer, copied with one
// transfer each way and unpacked; device operands are used in place.
int gb_dgemm_batch_grouped(int order, const int *ta, const int *tb, const blasint *m,
                           const blasint *n, const blasint *k, const double *alpha,
                           const double **A, const blasint *lda, const double **B,
                           const blasint *ldb, const double *beta, double **C,
                           const blasint *ldc, blasint group_count, const blasint *group_size) {
  int st = ensure_init();
  if (st) return st;
  cudaStream_t s = stream();
  const bool row = order == CblasRowMajor;
  int64_t total = 0;
  for (blasint g = 0; g < group_count; ++g) total += group_size[g];
  if (total == 0) return GB_SUCCESS;
  // device or host operands (decided on the first problem, applied to all)
  const double *firstA = nullptr;
  for (blasint g = 0, idx = 0; g < group_count && !firstA; idx += group_size[g], ++g)
    if (group_size[g] > 0) firstA = C[idx];
  const bool on_device = firstA && is_device_pointer(firstA);
  std::vector<gb_batch_problem> probs;
  probs.reserve((size_t)total);
  // host staging: offsets of every packed operand
  struct Pack {
    const double *src;
    double *dst_host;
    int64_t rows, cols, ld;
    size_t off;
    bool out;
  };
  std::vector<Pack> packs;
  size_t elems = 0;
  auto add = [&](const double *src, int64_t rows, int64_t cols, int64_t ld, bool out) {
    Pack pk{src, const_cast<double *>(src), rows, cols, ld, elems, out};
    packs.push_back(pk);
    elems += (size_t)rows * cols;
    return packs.size() - 1;
  };
  std::vector<size_t> pa, pb, pc;
  int64_t idx = 0;
  for (blasint g = 0; g < group_count; ++g) {
    const int64_t M = row ? n[g] : m[g], N = row ? m[g] : n[g], K = k[g];
    for (blasint t = 0; t < group_size[g]; ++t, ++idx) {
      gb_batch_problem p;
      memset(&p, 0, sizeof(p));
      p.type = GB_BATCH_DGEMM;
      p.m = (int)M;
      p.n = (int)N;
      p.k = (int)K;
      p.transa = ta[g] ? 'T' : 'N';
      p.transb = tb[g] ? 'T' : 'N';
      p.alpha = alpha[g];
      p.beta = beta[g];
      const double *pa_ = row ? B[idx] : A[idx];
      const double *pb_ = row ? A[idx] : B[idx];
      p.lda = (int)(row ? ldb[g] : lda[g]);
      p.ldb = (int)(row ? lda[g] : ldb[g]);
      p.ldc = (int)ldc[g];
      p.A = const_cast<double *>(pa_);
      p.B = const_cast<double *>(pb_);
      p.C = C[idx];
      if (M == 0 || N == 0) continue;
      if (!on_device) {
        const bool need_ab = K > 0 && alpha[g] != 0.0;
        const int64_t ra = ta[g] ? K : M, ca = ta[g] ? M : K;
        const int64_t rb = tb[g] ? N : K, cb = tb[g] ? K : N;
        pa.push_back(need_ab ? add(pa_, ra, ca, p.lda, false) : (size_t)-1);
        pb.push_back(need_ab ? add(pb_, rb, cb, p.ldb, false) : (size_t)-1);
        pc.push_back(add(C[idx], M, N, p.ldc, true));
      }
      probs.push_back(p);
    }
  }
  Scratch dev(on_device ? 0 : elems * sizeof(double), s);
  // the pinned staging buffer and the plan, released on every return path
  struct Held {
    double *hbuf = nullptr;
    void *plan = nullptr;
    ~Held() {
      if (plan) gb_batch_plan_destroy(plan);
      if (hbuf) cudaFreeHost(hbuf);
    }
  } held;
  double *&hbuf = held.hbuf;
  if (!on_device) {
    if (!dev.p) return GB_ERR_ALLOC;
    GB_CUDA(cudaMallocHost((void **)&hbuf, elems * sizeof(double)));
    for (const Pack &pk : packs)
      for (int64_t c = 0; c < pk.cols; ++c)
        memcpy(hbuf + pk.off + c * pk.rows, pk.src + c * pk.ld, pk.rows * sizeof(double));
    GB_CUDA(cudaMemcpyAsync(dev.p, hbuf, elems * sizeof(double), cudaMemcpyHostToDevice, s));
    double *d = dev.as<double>();
    for (size_t i = 0; i < probs.size(); ++i) {
      gb_batch_problem &p = probs[i];
      if (pa[i] != (size_t)-1) {
        p.A = d + packs[pa[i]].off;
        p.lda = (int)packs[pa[i]].rows;
        p.B = d + packs[pb[i]].off;
        p.ldb = (int)packs[pb[i]].rows;
      }
      p.C = d + packs[pc[i]].off;
      p.ldc = (int)packs[pc[i]].rows;
      if (p.ldc < 1) p.ldc = 1;
      if (p.lda < 1) p.lda = 1;
      if (p.ldb < 1) p.ldb = 1;
    }
  }
  void *plan = held.plan = gb_batch_plan_create(probs.data(), (int)probs.size(), 0);
  if (!plan) return GB_ERR_CUDA;
  st = gb_batch_execute(plan);
  if (!st && !on_device) {
    GB_CUDA(cudaMemcpyAsync(hbuf, dev.p, elems * sizeof(double), cudaMemcpyDeviceToHost, s));
    st = finish_blocking(s);
    if (!st)
      for (const Pack &pk : packs)
        if (pk.out)
          for (int64_t c = 0; c < pk.cols; ++c)
            memcpy(pk.dst_host + c * pk.ld, hbuf + pk.off + c * pk.rows, pk.rows * sizeof(double));
  } else if (!st) {
    st = finish_blocking(s);
  }
  return st;
}

}  // namespace gb

extern "C" {

void gb_batch_plan_destroy(void *plan) {
  BatchPlan *pl = reinterpret_cast<BatchPlan *>(plan);
  if (!pl) return;
  if (pl->exec) cudaGraphExecDestroy(pl->exec);
  if (pl->graph) cudaGraphDestroy(pl->graph);
  cudaFree(pl->d_probs);
  cudaFree(pl->d_order);
  cudaFree(pl->d_order_emu);
  cudaFree(pl->d_next);
  cudaFree(pl->d_work);
  cudaFree(pl->d_loopnext);
  delete pl;
}

}  // extern "C"
