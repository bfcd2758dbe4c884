// Complex GEMM -- ZGEMM/CGEMM and the 3M forms ZGEMM3M/CGEMM3M -- on the
// real GEMM engines (native DFMA or emulated FP64 for Z, the bf16x3 tensor
// form or FFMA for C).
//
// Semantics follow interface/gemm.c compiled with COMPLEX (op codes N = 0,
// T = 1, R = 2 conjugate without transpose, C = 3 conjugate transpose,
// gemm.c:253-268), driver/level3/level3.c:229-259 (C = beta C first, unless
// beta = 1; nothing more when k = 0 or alpha = 0) and
// kernel/generic/zgemm_beta.c:38-100 (beta = 0 stores zeros, so NaN in C is
// overwritten).
//
// 4M (ZGEMM, CGEMM).  The complex product is one real GEMM on an embedding:
//     op(A) op(B) = [Ar -Ai; Ai Ar] [Br; Bi]   (2m x 2k times 2k x n)
// whose 2m x n result P holds Re over Im.  The embeddings are built in the
// stored layout of A and B (a transposed operand is embedded transposed and
// handed to the real GEMM with its transpose flag), so every copy kernel reads
// and writes along columns.  The epilogue forms C = beta C + alpha P with the
// complex scaling of the reference's kernels (zgemmkernel_2x2.c: alpha applied
// to the accumulated sums).  Real flops: 8mnk, as in a complex kernel.
//
// 3M (ZGEMM3M, CGEMM3M), driver/level3/gemm3m_level3.c: alpha is folded
// into the copies of B (zgemm3m_ncopy_*.c: B' = alpha op(B) with
// Re = ar*br - ai*bi, Im = ai*br + ar*bi), then three real products
//     T1 = (Ar + Ai)(B'r + B'i),  T2 = Ar B'r,  T3 = Ai B'i
// and Re(C) += T2 - T3, Im(C) += T1 - T2 - T3 after C = beta C.  Real flops:
// 6mnk.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_internal.h"
#include "lapack_internal.h"

namespace gb {

namespace {

unsigned grid_for(int64_t total) {
  const int64_t blocks = (total + 255) / 256, cap = (int64_t)sm_count() * 16;
  return (unsigned)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

// E (2R x 2W, leading dimension 2R) from the complex R x W matrix X:
//   [ Xr       s_tr*Xi ]
//   [ s_bl*Xi  Xr      ]
template <typename T>
__global__ void embed4_kernel(int64_t R, int64_t W, const T *__restrict__ X, int64_t ldx,
                              T s_tr, T s_bl, T *__restrict__ E) {
  const int64_t total = R * W, ld = 2 * R;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / R, i = e - j * R;
    const T xr = X[2 * (i + j * ldx)], xi = X[2 * (i + j * ldx) + 1];
    E[i + j * ld] = xr;
    E[R + i + j * ld] = s_bl * xi;
    E[i + (W + j) * ld] = s_tr * xi;
    E[R + i + (W + j) * ld] = xr;
  }
}

// F from the complex R x W matrix Y: [Yr; t*Yi] (2R x W, leading dimension
// 2R) when `vertical`, else [Yr, t*Yi] (R x 2W, leading dimension R).
template <typename T>
__global__ void stack2_kernel(int64_t R, int64_t W, const T *__restrict__ Y, int64_t ldy, T t,
                              int vertical, T *__restrict__ F) {
  const int64_t total = R * W;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / R, i = e - j * R;
    const T yr = Y[2 * (i + j * ldy)], yi = Y[2 * (i + j * ldy) + 1];
    if (vertical) {
      F[i + j * 2 * R] = yr;
      F[R + i + j * 2 * R] = t * yi;
    } else {
      F[i + j * R] = yr;
      F[i + (W + j) * R] = t * yi;
    }
  }
}

// The three real R x W operands of the 3M product (leading dimension R):
// v = X or conj(X); with `scale`, w = alpha v (zgemm3m_ncopy_*.c REAL_PART /
// IMAGE_PART), else w = v; out = [wr, wi, wr + wi].
template <typename T>
__global__ void split3m_kernel(int64_t R, int64_t W, const T *__restrict__ X, int64_t ldx,
                               int conj, int scale, T ar, T ai, T *__restrict__ out) {
  const int64_t total = R * W;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / R, i = e - j * R;
    const T vr = X[2 * (i + j * ldx)];
    const T vi = conj ? -X[2 * (i + j * ldx) + 1] : X[2 * (i + j * ldx) + 1];
    T wr = vr, wi = vi;
    if (scale) {
      wr = ar * vr - ai * vi;
      wi = ai * vr + ar * vi;
    }
    out[e] = wr;
    out[total + e] = wi;
    out[2 * total + e] = wr + wi;
  }
}

// c <- beta c as zgemm_beta.c: zeros for beta = 0, untouched for beta = 1.
template <typename T>
__device__ __forceinline__ void scale_beta(T &cr, T &ci, T br, T bi) {
  if (br == T(0) && bi == T(0)) {
    cr = T(0);
    ci = T(0);
  } else if (!(br == T(1) && bi == T(0))) {
    const T r = br * cr - bi * ci, i = br * ci + bi * cr;
    cr = r;
    ci = i;
  }
}

// mode 0: C = beta C; mode 1 (4M): C = beta C + alpha P, P = [Re; Im] with
// leading dimension 2m; mode 2 (3M): Re += T2 - T3, Im += T1 - T2 - T3 on
// the three m x n products stored back to back.
template <typename T>
__global__ void complex_epilogue_kernel(int64_t m, int64_t n, int mode, T ar, T ai,
                                        const T *__restrict__ P, T br, T bi, T *__restrict__ C,
                                        int64_t ldc) {
  const int64_t total = m * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / m, i = e - j * m;
    T *c = C + 2 * (i + j * ldc);
    T cr = c[0], ci = c[1];
    scale_beta(cr, ci, br, bi);
    if (mode == 1) {
      const T pr = P[i + j * 2 * m], pi = P[m + i + j * 2 * m];
      cr += ar * pr - ai * pi;
      ci += ar * pi + ai * pr;
    } else if (mode == 2) {
      const T t1 = P[e], t2 = P[total + e], t3 = P[2 * total + e];
      ci += t1;
      cr += t2;
      ci -= t2;
      cr -= t3;
      ci -= t3;
    }
    c[0] = cr;
    c[1] = ci;
  }
}

// C = op(A) op(B) on the real engine of the type (alpha 1, beta 0).
int real_gemm(int ta, int tb, int64_t m, int64_t n, int64_t k, const double *A, int64_t lda,
              const double *B, int64_t ldb, double *C, int64_t ldc, cudaStream_t s) {
  return dgemm_select(ta, tb, m, n, k, 1.0, A, lda, B, ldb, 0.0, C, ldc, 0, s);
}
int real_gemm(int ta, int tb, int64_t m, int64_t n, int64_t k, const float *A, int64_t lda,
              const float *B, int64_t ldb, float *C, int64_t ldc, cudaStream_t s) {
  return sgemm_dispatch(ta, tb, m, n, k, 1.0f, A, lda, B, ldb, 0.0f, C, ldc, s);
}

}  // namespace

// C = alpha op(A) op(B) + beta C for complex T pairs (interleaved re, im),
// ta/tb in 0..3 (N, T, R, C), alpha/beta host pointers to (re, im);
// three_m selects the 3M product.
template <typename T>
int cgemm_device(int ta, int tb, int64_t m, int64_t n, int64_t k, const T *alpha, const T *A,
                 int64_t lda, const T *B, int64_t ldb, const T *beta, T *C, int64_t ldc,
                 int three_m, cudaStream_t s) {
  if (m == 0 || n == 0) return GB_SUCCESS;
  const T ar = alpha[0], ai = alpha[1], br = beta[0], bi = beta[1];
  if (k == 0 || (ar == T(0) && ai == T(0))) {
    if (br == T(1) && bi == T(0)) return GB_SUCCESS;
    complex_epilogue_kernel<T><<<grid_for(m * n), 256, 0, s>>>(m, n, 0, ar, ai, nullptr, br,
                                                                  bi, C, ldc);
    count_launch();
    return check_cuda(cudaGetLastError(), "complex gemm beta");
  }
  const int tA = ta & 1, tB = tb & 1;
  const bool cA = ta >= 2, cB = tb >= 2;
  const int64_t ra = tA ? k : m, ca = tA ? m : k;  // A as stored
  const int64_t rb = tB ? n : k, cb = tB ? k : n;  // B as stored
  int st;
  if (!three_m) {
    Scratch ws((size_t)(4 * m * k + 2 * k * n + 2 * m * n) * sizeof(T), s);
    if (!ws.p) return GB_ERR_ALLOC;
    T *E = ws.as<T>(), *F = E + 4 * m * k, *P = F + 2 * k * n;
    const T sg = cA ? T(-1) : T(1);
    // transposed A is embedded as [Xr, s Xi; -s Xi, Xr], so that its transpose
    // is [Ar -Ai; Ai Ar] of op(A)
    { embed4_kernel<T><<<grid_for(ra * ca), 256, 0, s>>>(ra, ca, A, lda, tA ? sg : -sg,
                                                             tA ? -sg : sg, E); count_launch(); }
    { stack2_kernel<T><<<grid_for(rb * cb), 256, 0, s>>>(rb, cb, B, ldb, cB ? T(-1) : T(1),
                                                             tB ? 0 : 1, F); count_launch(); }
    if ((st = check_cuda(cudaGetLastError(), "complex gemm embed"))) return st;
    if ((st = real_gemm(tA, tB, 2 * m, n, 2 * k, E, 2 * ra, F, tB ? rb : 2 * rb, P, 2 * m, s)))
      return st;
    { complex_epilogue_kernel<T><<<grid_for(m * n), 256, 0, s>>>(m, n, 1, ar, ai, P, br, bi,
                                                                     C, ldc); count_launch(); }
    return check_cuda(cudaGetLastError(), "complex gemm epilogue");
  }
  Scratch ws((size_t)3 * (m * k + k * n + m * n) * sizeof(T), s);
  if (!ws.p) return GB_ERR_ALLOC;
  T *XA = ws.as<T>(), *YB = XA + 3 * m * k, *TP = YB + 3 * k * n;
  { split3m_kernel<T><<<grid_for(ra * ca), 256, 0, s>>>(ra, ca, A, lda, cA ? 1 : 0, 0, T(1),
                                                            T(0), XA); count_launch(); }
  { split3m_kernel<T><<<grid_for(rb * cb), 256, 0, s>>>(rb, cb, B, ldb, cB ? 1 : 0, 1, ar, ai,
                                                            YB); count_launch(); }
  if ((st = check_cuda(cudaGetLastError(), "complex gemm 3m split"))) return st;
  const int64_t sa = m * k, sb = k * n, sc = m * n;
  // T1 = (Ar + Ai)(B'r + B'i), T2 = Ar B'r, T3 = Ai B'i
  if ((st = real_gemm(tA, tB, m, n, k, XA + 2 * sa, ra, YB + 2 * sb, rb, TP, m, s))) return st;
  if ((st = real_gemm(tA, tB, m, n, k, XA, ra, YB, rb, TP + sc, m, s))) return st;
  if ((st = real_gemm(tA, tB, m, n, k, XA + sa, ra, YB + sb, rb, TP + 2 * sc, m, s))) return st;
  { complex_epilogue_kernel<T><<<grid_for(m * n), 256, 0, s>>>(m, n, 2, ar, ai, TP, br, bi, C,
                                                                   ldc); count_launch(); }
  return check_cuda(cudaGetLastError(), "complex gemm 3m epilogue");
}

template int cgemm_device<double>(int, int, int64_t, int64_t, int64_t, const double *,
                                  const double *, int64_t, const double *, int64_t,
                                  const double *, double *, int64_t, int, cudaStream_t);
template int cgemm_device<float>(int, int, int64_t, int64_t, int64_t, const float *,
                                 const float *, int64_t, const float *, int64_t, const float *,
                                 float *, int64_t, int, cudaStream_t);

}  // namespace gb
