// Native FP64 (DFMA) and FP32 (FFMA) GEMM kernels and the beta-scaling
// kernel of libgbblas.
//
// Semantics follow driver/level3/level3.c:229-259 and
// kernel/generic/gemm_beta.c:41-94: C <- beta*C first (beta==0 stores zeros,
// so NaNs in C are not propagated), nothing more when k==0 or alpha==0,
// otherwise C += alpha*op(A)*op(B).  The kernels fuse the beta pass into the
// epilogue: C = alpha*acc + beta*C, reading C only when beta != 0.
//
// GB300 has no FP64 tensor-core kind (tcgen05 has none, and mma.sync f64
// measures slower than DFMA on this part), so the native FP64 GEMM is a
// register-tiled DFMA kernel.  With ~2 DFMA/clock/SM the kernel is bound by
// the FP64 pipe; a 64x64 tile (4x4 per thread) already needs only ~0.5 B/clk
// of operand traffic per SM.  Grids are sized so every SM gets an even share
// (32x32 tiles when 64x64 would leave SMs idle).
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_internal.h"

namespace gb {
namespace {

template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__(256)
gemm_simt_kernel(int ta, int tb, int64_t m, int64_t n, int64_t k, T alpha,
                 const T *__restrict__ A, int64_t lda, const T *__restrict__ B,
                 int64_t ldb, T beta, T *__restrict__ C, int64_t ldc, int tri,
                 const int *__restrict__ skip) {
  constexpr int TX = BM / TM;  // threads along M
  constexpr int TY = BN / TN;  // threads along N
  static_assert(TX * TY == 256, "256 threads");
  constexpr int LA = BM * BK / 256;  // elements of A tile per thread
  constexpr int LB = BN * BK / 256;
  static_assert(LA * 256 == BM * BK && LB * 256 == BN * BK, "tile split");

  __shared__ T As[2][BK][BM];
  __shared__ T Bs[2][BK][BN];

  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  // tri: 0 full C, 1 lower triangle only (i >= j), 2 upper only (i <= j)
  if (tri == 1 && m0 + BM - 1 < n0) return;
  // skip: optional device flag (a factorisation's info) that cancels the update
  if (skip && *skip) return;
  if (tri == 2 && m0 > n0 + BN - 1) return;

  T ra[LA], rb[LB];
  auto load_tiles = [&](int64_t k0) {
#pragma unroll
    for (int t = 0; t < LA; ++t) {
      int e = tid + t * 256;
      int i, kk;
      if (!ta) { i = e % BM; kk = e / BM; }
      else     { kk = e % BK; i = e / BK; }
      int64_t gi = m0 + i, gk = k0 + kk;
      T v = T(0);
      if (gi < m && gk < k) v = ta ? A[gk + gi * lda] : A[gi + gk * lda];
      ra[t] = v;
    }
#pragma unroll
    for (int t = 0; t < LB; ++t) {
      int e = tid + t * 256;
      int j, kk;
      if (!tb) { kk = e % BK; j = e / BK; }
      else     { j = e % BN; kk = e / BN; }
      int64_t gj = n0 + j, gk = k0 + kk;
      T v = T(0);
      if (gj < n && gk < k) v = tb ? B[gj + gk * ldb] : B[gk + gj * ldb];
      rb[t] = v;
    }
  };
  auto store_tiles = [&](int buf) {
#pragma unroll
    for (int t = 0; t < LA; ++t) {
      int e = tid + t * 256;
      int i, kk;
      if (!ta) { i = e % BM; kk = e / BM; }
      else     { kk = e % BK; i = e / BK; }
      As[buf][kk][i] = ra[t];
    }
#pragma unroll
    for (int t = 0; t < LB; ++t) {
      int e = tid + t * 256;
      int j, kk;
      if (!tb) { kk = e % BK; j = e / BK; }
      else     { j = e % BN; kk = e / BN; }
      Bs[buf][kk][j] = rb[t];
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

  const int64_t ktiles = (k + BK - 1) / BK;
  load_tiles(0);
  store_tiles(0);
  __syncthreads();
  for (int64_t kt = 0; kt < ktiles; ++kt) {
    const int buf = (int)(kt & 1);
    if (kt + 1 < ktiles) load_tiles((kt + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[buf][kk][tx + i * TX];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[buf][kk][ty + j * TY];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    if (kt + 1 < ktiles) store_tiles(buf ^ 1);
    __syncthreads();
  }

#pragma unroll
  for (int j = 0; j < TN; ++j) {
    int64_t gj = n0 + ty + j * TY;
    if (gj >= n) continue;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      int64_t gi = m0 + tx + i * TX;
      if (gi >= m) continue;
      if ((tri == 1 && gi < gj) || (tri == 2 && gi > gj)) continue;
      T *c = C + gi + gj * ldc;
      T v = alpha * acc[i][j];
      if (beta != T(0)) v = fma(beta, *c, v);
      *c = v;
    }
  }
}

template <typename T>
__global__ void gemm_beta_kernel(int64_t m, int64_t n, T beta, T *__restrict__ C, int64_t ldc,
                                 int tri) {
  const int64_t total = m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t j = e / m, i = e - j * m;
    if ((tri == 1 && i < j) || (tri == 2 && i > j)) continue;
    T *c = C + i + j * ldc;
    *c = (beta == T(0)) ? T(0) : beta * *c;
  }
}

}  // namespace

int sm_count() {
  static PerDeviceValue<int> cache;
  const int dev = current_device();
  return cache.get(dev, [dev] {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      n = 0;
    }
    return n > 0 ? n : 152;
  });
}

void launch_dgemm_beta(int64_t m, int64_t n, double beta, double *C, int64_t ldc,
                       cudaStream_t s) {
  if (m <= 0 || n <= 0 || beta == 1.0) return;
  int64_t blocks = (m * n + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  { gemm_beta_kernel<double><<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(m, n, beta,
                                                                                  C, ldc, 0); count_launch(); }
}

void launch_sgemm_beta(int64_t m, int64_t n, float beta, float *C, int64_t ldc,
                       cudaStream_t s) {
  if (m <= 0 || n <= 0 || beta == 1.0f) return;
  int64_t blocks = (m * n + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  { gemm_beta_kernel<float><<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(m, n, beta, C,
                                                                                 ldc, 0); count_launch(); }
}

void launch_dgemm_fp64_tri(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                           const double *A, int64_t lda, const double *B, int64_t ldb,
                           double beta, double *C, int64_t ldc, int tri, cudaStream_t s,
                           const int *skip) {
  if (n > GEMM_BLOCK_EXTENT && tri == 0) {  // column tiles sit on gridDim.y
    gemm_over_blocks(ta, tb, m, n, A, lda, B, ldb, C, ldc, GEMM_BLOCK_EXTENT,
                     [&](int64_t mb, int64_t nb, const double *Ai, const double *Bj,
                         double *Cij) {
                       launch_dgemm_fp64_tri(ta, tb, mb, nb, k, alpha, Ai, lda, Bj, ldb, beta,
                                             Cij, ldc, 0, s, skip);
                       return 0;
                     });
    return;
  }
  ProfileScope prof("dgemm_fp64", s);
  const int64_t tiles64 = ((m + 63) / 64) * ((n + 63) / 64);
  if (tiles64 >= (int64_t)sm_count() * 8) {
    dim3 grid((unsigned)((m + 63) / 64), (unsigned)((n + 63) / 64));
    { gemm_simt_kernel<double, 64, 64, 16, 4, 4><<<grid, 256, 0, s>>>(
        ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, skip); count_launch(); }
  } else if (((m + 31) / 32) * ((n + 31) / 32) >= (int64_t)sm_count()) {
    dim3 grid((unsigned)((m + 31) / 32), (unsigned)((n + 31) / 32));
    { gemm_simt_kernel<double, 32, 32, 16, 2, 2><<<grid, 256, 0, s>>>(
        ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, skip); count_launch(); }
  } else {
    // fewer 32 x 32 tiles than SMs (the Cholesky's in-block updates): 16 x 16
    // tiles spread the FP64 work, which one SM does at ~2 FMA per clock
    dim3 grid((unsigned)((m + 15) / 16), (unsigned)((n + 15) / 16));
    { gemm_simt_kernel<double, 16, 16, 16, 1, 1><<<grid, 256, 0, s>>>(
        ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, skip); count_launch(); }
  }
}

void launch_dgemm_fp64(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                       const double *A, int64_t lda, const double *B, int64_t ldb, double beta,
                       double *C, int64_t ldc, cudaStream_t s) {
  launch_dgemm_fp64_tri(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, 0, s, nullptr);
}

void launch_dbeta_tri(int64_t n, double beta, double *C, int64_t ldc, int tri, cudaStream_t s) {
  if (n <= 0 || beta == 1.0) return;
  int64_t blocks = (n * n + 255) / 256;
  int64_t cap = (int64_t)sm_count() * 16;
  { gemm_beta_kernel<double><<<(unsigned)(blocks < cap ? blocks : cap), 256, 0, s>>>(n, n, beta,
                                                                                  C, ldc, tri); count_launch(); }
}

void launch_sgemm_fp32_tri(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha,
                           const float *A, int64_t lda, const float *B, int64_t ldb, float beta,
                           float *C, int64_t ldc, int tri, cudaStream_t s, const int *skip) {
  if (n > GEMM_BLOCK_EXTENT && tri == 0) {  // column tiles sit on gridDim.y
    gemm_over_blocks(ta, tb, m, n, A, lda, B, ldb, C, ldc, GEMM_BLOCK_EXTENT,
                     [&](int64_t mb, int64_t nb, const float *Ai, const float *Bj, float *Cij) {
                       launch_sgemm_fp32_tri(ta, tb, mb, nb, k, alpha, Ai, lda, Bj, ldb, beta,
                                             Cij, ldc, 0, s, skip);
                       return 0;
                     });
    return;
  }
  const int64_t tiles128 = ((m + 127) / 128) * ((n + 127) / 128);
  if (tiles128 >= (int64_t)sm_count() * 2) {
    dim3 grid((unsigned)((m + 127) / 128), (unsigned)((n + 127) / 128));
    { gemm_simt_kernel<float, 128, 128, 8, 8, 8><<<grid, 256, 0, s>>>(
        ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, skip); count_launch(); }
  } else {
    dim3 grid((unsigned)((m + 63) / 64), (unsigned)((n + 63) / 64));
    { gemm_simt_kernel<float, 64, 64, 16, 4, 4><<<grid, 256, 0, s>>>(
        ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri, skip); count_launch(); }
  }
}

void launch_sgemm_fp32(int ta, int tb, int64_t m, int64_t n, int64_t k, float alpha,
                       const float *A, int64_t lda, const float *B, int64_t ldb, float beta,
                       float *C, int64_t ldc, cudaStream_t s) {
  launch_sgemm_fp32_tri(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, 0, s, nullptr);
}

}  // namespace gb
