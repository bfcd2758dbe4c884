// A GEMM run as a sequence of GEMMs on blocks of C.
//
// Several launches here put a row or column count of C on gridDim.y, which
// CUDA caps at 65535: the slice and bf16x3 split kernels (32 rows of op(A) or
// columns of op(B) per block) and the FP64/FP32 SIMT GEMMs (one column tile
// per block).  The emulated engine's scratch also grows with m and n.  A
// GEMM whose m or n exceeds GEMM_BLOCK_EXTENT therefore runs block by block
// over C.  Element C(i, j) depends only on row i of op(A) and column j of
// op(B), and every engine here computes it from exactly those: the emulated
// engine's exponents are per row of op(A) and per column of op(B), and the
// bf16x3 engine's Inf/NaN rows and columns are flagged the same way.  So
// each element sees the same data as in a single call.  This header needs no
// CUDA headers.
#pragma once

#include <stdint.h>

namespace gb {

constexpr int64_t GEMM_BLOCK_EXTENT = int64_t(1) << 20;

// Calls gemm(mb, nb, A_i, B_j, C_ij) on each block of C with at most `extent`
// rows and columns, rows outermost, and returns the first non-zero status.
// ta / tb: bit 0 set when op(X) is X transposed (conjugate forms included),
// so a block's op(A) rows start at A + i0 * lda and its op(B) columns at
// B + j0 (otherwise A + i0 and B + j0 * ldb).
template <typename T, typename F>
int gemm_over_blocks(int ta, int tb, int64_t m, int64_t n, const T *A, int64_t lda, const T *B,
                     int64_t ldb, T *C, int64_t ldc, int64_t extent, F &&gemm) {
  for (int64_t i0 = 0; i0 < m; i0 += extent) {
    const int64_t mb = m - i0 < extent ? m - i0 : extent;
    const T *Ai = (ta & 1) ? A + i0 * lda : A + i0;
    for (int64_t j0 = 0; j0 < n; j0 += extent) {
      const int64_t nb = n - j0 < extent ? n - j0 : extent;
      const T *Bj = (tb & 1) ? B + j0 : B + j0 * ldb;
      const int st = gemm(mb, nb, Ai, Bj, C + i0 + j0 * ldc);
      if (st) return st;
    }
  }
  return 0;
}

}  // namespace gb
