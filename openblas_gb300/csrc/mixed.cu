// Mixed-precision linear solve: FP32 LU on the GPU, FP64 iterative
// refinement, GMRES-IR when plain refinement stalls, FP64 LU as the last
// resort.
//
// The outer algorithm restates lapack-netlib/SRC/dsgesv.f:193-430:
//   anrm = ||A||_inf, cte = anrm * eps * sqrt(n)   (eps = 2^-53)
//   SA = fp32(A), SX = fp32(B)  (overflow -> ITER = -2, FP64 fallback)
//   sgetrf(SA) (singular -> ITER = -3, FP64 fallback), SX = sgetrs(SX)
//   X = fp64(SX); repeat up to 30 times:
//     R = B - A X (FP64); stop when max|R(:,j)| <= max|X(:,j)| * cte for all j
//     X += fp64(sgetrs(fp32(R)))
//   no convergence -> ITER = -31, FP64 dgetrf + dgetrs.
// The GMRES-IR stage (not in the reference; Carson & Higham, SIAM J. Sci.
// Comput. 2018) is entered when the refinement stops contracting: for each
// right-hand side, restarted flexible GMRES in FP64 on A d = r with the FP32
// LU as right preconditioner, then x += d and the same stopping test.  It
// finishes ill-conditioned solves whose FP32 factors precondition all but a
// few directions: with 8 singular values at 1e-8 or 1e-12 (the rest 1) it
// converges in 15-25 iterations at n = 4096 and 8192.  Where the small
// singular values fill a large part of the spectrum (U diag(logspace(0,-8))
// V^T) no FP32 factorisation preconditions them; the first restart cycle
// shows it and the solve goes to the FP64-accurate LU (emulated-FP64
// trailing updates).  The reported ITER is 100 + (GMRES iterations) when
// GMRES-IR finishes the solve.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "gb_internal.h"
#include "lapack_internal.h"
#include "operand.h"

namespace gb {


namespace {

constexpr int GEMV_COL_CHUNK = 256;

// ||A||_inf partial row sums over column chunks: part[chunk][i]
__global__ void absrowsum_kernel(int64_t m, int64_t n, const double *__restrict__ A, int64_t lda,
                                 int64_t chunk, double *__restrict__ part) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int64_t j0 = (int64_t)blockIdx.y * chunk, j1 = j0 + chunk < n ? j0 + chunk : n;
  double s = 0.0;
  for (int64_t j = j0; j < j1; ++j) s += fabs(A[i + j * lda]);
  part[(int64_t)blockIdx.y * m + i] = s;
}

// out = max over rows of the summed partials (single block)
__global__ void rowsum_max_kernel(int64_t m, int nchunks, const double *__restrict__ part,
                                  double *__restrict__ out) {
  __shared__ double red[256];
  double best = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nchunks; ++c) s += part[(int64_t)c * m + i];
    if (s > best || isnan(s)) best = s;
  }
  red[threadIdx.x] = best;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double o = red[threadIdx.x + w];
      if (o > red[threadIdx.x] || isnan(o)) red[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// FP64 -> FP32 with the overflow test of dlag2s.f:136-145
__global__ void lag2s_kernel(int64_t m, int64_t n, const double *__restrict__ A, int64_t lda,
                             float *__restrict__ S, int64_t lds, int *__restrict__ flag) {
  const int64_t total = m * n;
  const double rmax = (double)FLT_MAX;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / m, i = e - j * m;
    const double v = A[i + j * lda];
    if (v < -rmax || v > rmax) *flag = 1;
    S[i + j * lds] = (float)v;
  }
}

// A = fp64(S) (accumulate = 0) or A += fp64(S)
__global__ void lag2d_kernel(int64_t m, int64_t n, const float *__restrict__ S, int64_t lds,
                             double *__restrict__ A, int64_t lda, int accumulate) {
  const int64_t total = m * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / m, i = e - j * m;
    const double v = (double)S[i + j * lds];
    if (accumulate)
      A[i + j * lda] += v;
    else
      A[i + j * lda] = v;
  }
}

// max_i |X(i,j)| per column (one block per column), IDAMAX magnitude
__global__ void colabsmax_kernel(int64_t m, const double *__restrict__ X, int64_t ldx,
                                 double *__restrict__ out) {
  __shared__ double red[256];
  const double *x = X + (int64_t)blockIdx.x * ldx;
  double best = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    const double a = fabs(x[i]);
    if (a > best || isnan(a)) best = a;
  }
  red[threadIdx.x] = best;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double o = red[threadIdx.x + w];
      if (o > red[threadIdx.x] || isnan(o)) red[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// y = B - A x for one column: partial sums over column chunks of A, then a
// combine pass.  A is read once, coalesced along rows.
__global__ void gemv_partial_kernel(int64_t n, const double *__restrict__ A, int64_t lda,
                                    const double *__restrict__ x, double *__restrict__ part) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t j0 = (int64_t)blockIdx.y * GEMV_COL_CHUNK;
  const int64_t j1 = j0 + GEMV_COL_CHUNK < n ? j0 + GEMV_COL_CHUNK : n;
  __shared__ double xs[GEMV_COL_CHUNK];
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) xs[j - j0] = x[j];
  __syncthreads();
  if (i >= n) return;
  double s0 = 0.0, s1 = 0.0;
  int64_t j = j0;
  for (; j + 1 < j1; j += 2) {
    s0 = fma(A[i + j * lda], xs[j - j0], s0);
    s1 = fma(A[i + (j + 1) * lda], xs[j + 1 - j0], s1);
  }
  if (j < j1) s0 = fma(A[i + j * lda], xs[j - j0], s0);
  part[(int64_t)blockIdx.y * n + i] = s0 + s1;
}

__global__ void gemv_combine_kernel(int64_t n, int nchunks, const double *__restrict__ part,
                                    double alpha, const double *__restrict__ b, double beta,
                                    double *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int c = 0; c < nchunks; ++c) s += part[(int64_t)c * n + i];
  y[i] = (beta == 0.0 ? 0.0 : beta * b[i]) + alpha * s;
}

// Compensated (double-double) form of the two kernels above, for the
// Krylov products of GMRES-IR: there z = M^-1 v has a norm near kappa(A)
// while A z is near v, so a plain FP64 product loses about n*eps*kappa of
// relative accuracy, which caps what GMRES can reach.  Each product a*x is
// split exactly with one FMA (TwoProduct) and the sums are carried as
// hi + lo with TwoSum, so the result is A z rounded once.
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  const double z = s - a;
  e = (a - (s - z)) + (b - z);
}

__global__ void gemv_dd_partial_kernel(int64_t n, const double *__restrict__ A, int64_t lda,
                                       const double *__restrict__ x, double *__restrict__ part_hi,
                                       double *__restrict__ part_lo) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t j0 = (int64_t)blockIdx.y * GEMV_COL_CHUNK;
  const int64_t j1 = j0 + GEMV_COL_CHUNK < n ? j0 + GEMV_COL_CHUNK : n;
  __shared__ double xs[GEMV_COL_CHUNK];
  for (int64_t j = j0 + threadIdx.x; j < j1; j += blockDim.x) xs[j - j0] = x[j];
  __syncthreads();
  if (i >= n) return;
  double hi = 0.0, lo = 0.0;
  for (int64_t j = j0; j < j1; ++j) {
    const double a = A[i + j * lda], b = xs[j - j0];
    const double p = a * b;
    const double pe = fma(a, b, -p);  // exact: a*b = p + pe
    double t, te;
    two_sum(hi, p, t, te);
    hi = t;
    lo += te + pe;
  }
  two_sum(hi, lo, hi, lo);
  part_hi[(int64_t)blockIdx.y * n + i] = hi;
  part_lo[(int64_t)blockIdx.y * n + i] = lo;
}

// y = beta*b + alpha*sum(parts), alpha = +-1 and beta in {0, 1} (exact), in
// double-double, rounded once.
__global__ void gemv_dd_combine_kernel(int64_t n, int nchunks, const double *__restrict__ part_hi,
                                       const double *__restrict__ part_lo, double alpha,
                                       const double *__restrict__ b, double beta,
                                       double *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double hi = beta == 0.0 ? 0.0 : beta * b[i], lo = 0.0;
  for (int c = 0; c < nchunks; ++c) {
    double t, te;
    two_sum(hi, alpha * part_hi[(int64_t)c * n + i], t, te);
    hi = t;
    lo += te + alpha * part_lo[(int64_t)c * n + i];
  }
  y[i] = hi + lo;
}

// out[j] = V(:,j) . w for j < k (one block per j)
__global__ void multidot_kernel(int64_t n, const double *__restrict__ V, int64_t ldv,
                                const double *__restrict__ w, double *__restrict__ out) {
  __shared__ double red[256];
  const double *v = V + (int64_t)blockIdx.x * ldv;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s = fma(v[i], w[i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// w -= V(:, 0:k) * h   (h on the device)
__global__ void multiaxpy_kernel(int64_t n, int k, const double *__restrict__ V, int64_t ldv,
                                 const double *__restrict__ h, double *__restrict__ w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = w[i];
  for (int j = 0; j < k; ++j) s = fma(-V[i + (int64_t)j * ldv], h[j], s);
  w[i] = s;
}

// y = a*x (+ y if accumulate)
__global__ void scale_kernel(int64_t n, double a, const double *__restrict__ x,
                             double *__restrict__ y, int accumulate) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  y[i] = accumulate ? fma(a, x[i], y[i]) : a * x[i];
}

unsigned grid_for(int64_t total, int64_t cap_per_sm = 16) {
  int64_t b = (total + 255) / 256;
  int64_t cap = (int64_t)sm_count() * cap_per_sm;
  return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
}

struct Host {
  double *p = nullptr;
  size_t n = 0;
  explicit Host(size_t cnt) : n(cnt) {
    if (cudaMallocHost((void **)&p, cnt * sizeof(double)) != cudaSuccess) p = nullptr;
  }
  ~Host() {
    if (p) cudaFreeHost(p);
  }
};

// Solver state shared by the refinement stages.
struct Mixed {
  int64_t n, nrhs;
  const double *A;
  int64_t lda;
  const double *B;
  int64_t ldb;
  double *X;
  int64_t ldx;
  int *ipiv;
  cudaStream_t s;
  float *SA = nullptr;   // n x n FP32 LU
  float *SX = nullptr;   // n x nrhs FP32 work
  double *R = nullptr;   // n x nrhs residual
  double *part = nullptr;
  int nchunks = 0;
  double *dnorm = nullptr;  // device scratch for norms
  int *dflag = nullptr;
  Host *hx = nullptr;       // pinned host scratch
  double *LU64 = nullptr;   // FP64 copy of the FP32 factors (GMRES-IR stage)
  double *Linv64 = nullptr, *Uinv64 = nullptr;  // its inverted 64x64 diagonal blocks
  double *W64 = nullptr;    // n-vector work of the FP64 preconditioner
  double *part_lo = nullptr;  // low parts of the compensated GEMV
  float *SX2 = nullptr;     // n x nrhs FP32 work (permuted right-hand sides)
  int *perm = nullptr;      // final row permutation of the FP32 LU
  bool chol = false;        // Cholesky factors (no interchanges, mirrored triangles)
  float *Linv = nullptr, *Uinv = nullptr;  // inverted 64x64 diagonal blocks of L, U

  // X32 = (LU)^-1 P * X32 (in place through SX2): the FP32 solve of the refinement
  int solve32(float *V, int64_t k) {
    static const bool trsm_solve = getenv("GB_MIXED_SOLVE") && !strcmp(getenv("GB_MIXED_SOLVE"), "trsm");
    int st;
    if (chol) {
      GB_CUDA(cudaMemcpyAsync(SX2, V, (size_t)n * k * sizeof(float), cudaMemcpyDeviceToDevice, s));
    } else {
      if (trsm_solve) return getrs_device<float>(0, n, k, SA, n, ipiv, V, n, s);
      if ((st = apply_perm<float>(n, k, perm, V, n, SX2, n, s))) return st;
    }
    if ((st = lu_block_solve<float>(n, k, SA, n, Linv, Uinv, SX2, n, s))) return st;
    GB_CUDA(cudaMemcpyAsync(V, SX2, (size_t)n * k * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return GB_SUCCESS;
  }

  // R = B - A X (FP64)
  int residual() {
    ProfileScope prof("mixed_residual", s);
    if (nrhs <= 8) {
      for (int64_t j = 0; j < nrhs; ++j) {
        dim3 g((unsigned)((n + 255) / 256), (unsigned)nchunks);
        { gemv_partial_kernel<<<g, 256, 0, s>>>(n, A, lda, X + j * ldx, part); count_launch(); }
        { gemv_combine_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, nchunks, part, -1.0, B + j * ldb, 1.0, R + j * n); count_launch(); }
      }
    } else {
      // many right-hand sides: the product runs on the emulated-FP64 GEMM, whose
      // error (a few eps * |A||X|) is the same scale as a native FP64 product's
      GB_CUDA(cudaMemcpy2DAsync(R, n * 8, B, ldb * 8, n * 8, nrhs, cudaMemcpyDeviceToDevice, s));
      int st = dgemm_emulated(0, 0, n, nrhs, n, -1.0, A, lda, X, ldx, 1.0, R, n, 0, s);
      if (st) return st;
    }
    return check_cuda(cudaGetLastError(), "residual");
  }

  // true when every column satisfies max|r| <= max|x| * cte (dsgesv.f:337-339)
  int converged(double cte, bool *ok, double *worst) {
    { colabsmax_kernel<<<(unsigned)nrhs, 256, 0, s>>>(n, X, ldx, dnorm); count_launch(); }
    { colabsmax_kernel<<<(unsigned)nrhs, 256, 0, s>>>(n, R, n, dnorm + nrhs); count_launch(); }
    GB_CUDA(cudaMemcpyAsync(hx->p, dnorm, 2 * nrhs * sizeof(double), cudaMemcpyDeviceToHost, s));
    int st = finish_blocking(s);
    if (st) return st;
    *ok = true;
    *worst = 0.0;
    for (int64_t j = 0; j < nrhs; ++j) {
      const double xn = hx->p[j], rn = hx->p[nrhs + j];
      if (!(rn <= xn * cte)) *ok = false;
      const double q = xn > 0 ? rn / xn : rn;
      if (q > *worst || isnan(q)) *worst = q;
    }
    return GB_SUCCESS;
  }

  // M^-1 v for GMRES-IR: the FP32 factors applied in FP64 arithmetic
  // v = (LU)^-1 P v with the FP64 copy of the FP32 factors: the chained
  // block solve (one launch per triangle), in place through W64
  int precond64(double *v) {
    int st = apply_perm<double>(n, 1, perm, v, n, W64, n, s);
    if (st) return st;
    if ((st = lu_block_solve<double>(n, 1, LU64, n, Linv64, Uinv64, W64, n, s))) return st;
    GB_CUDA(cudaMemcpyAsync(v, W64, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return GB_SUCCESS;
  }

  // y = beta*b + alpha*A*x in double-double (one column), for the Krylov products
  void gemv_dd(const double *x, double alpha, const double *b, double beta, double *y) {
    dim3 gg((unsigned)((n + 255) / 256), (unsigned)nchunks);
    { gemv_dd_partial_kernel<<<gg, 256, 0, s>>>(n, A, lda, x, part, part_lo); count_launch(); }
    { gemv_dd_combine_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, nchunks, part, part_lo, alpha, b, beta, y); count_launch(); }
  }

  // FP32 solve of the n x k block V (in place through SX): V = fp64(LU32 \ fp32(V))
  int precond(double *V, int64_t ldv, int64_t k, bool *overflow) {
    GB_CUDA(cudaMemsetAsync(dflag, 0, sizeof(int), s));
    { lag2s_kernel<<<grid_for(n * k), 256, 0, s>>>(n, k, V, ldv, SX, n, dflag); count_launch(); }
    int st;
    {
      ProfileScope prof("mixed_getrs", s);
      st = solve32(SX, k);
    }
    if (st) return st;
    { lag2d_kernel<<<grid_for(n * k), 256, 0, s>>>(n, k, SX, n, V, ldv, 0); count_launch(); }
    int h = 0;
    GB_CUDA(cudaMemcpyAsync(&hx->p[0], dflag, sizeof(int), cudaMemcpyDeviceToHost, s));
    if ((st = finish_blocking(s))) return st;
    memcpy(&h, &hx->p[0], sizeof(int));
    *overflow = h != 0;
    return GB_SUCCESS;
  }
};

// Restarted flexible GMRES for A d = r (one column), right preconditioner
// M^-1 = the FP32 LU.  Returns iterations used; d is written to `d`.  A first
// restart cycle whose 16th iteration has not reduced the residual tenfold,
// 16 consecutive iterations that do not halve it, or a cycle that does not
// reduce it a hundredfold, set *hopeless: at that rate the iteration budget
// cannot reach FP64 accuracy (measured on U diag(logspace(0,-8)) V^T at
// n = 4096 and 8192, where the FP32 factors leave a quarter of the spectrum
// unpreconditioned: a first cycle drops the residual ~7000x and then
// stalls, and the next cycle reduces it by less than 1%, while a matrix with
// a few tiny singular values converges within ~25 iterations).  The residual
// norm of each iterate is the Givens-rotated |g_j+1|, known on the host.
int fgmres(Mixed &M, const double *r, double *d, int restart, int max_it, double rtol,
           int *iters, bool *hopeless) {
  *hopeless = false;
  const int64_t n = M.n;
  cudaStream_t s = M.s;
  Scratch ws((size_t)n * (2 * restart + 2) * sizeof(double) + (restart + 2) * 16 + 256, s);
  if (!ws.p) return GB_ERR_ALLOC;
  double *V = ws.as<double>();               // n x (restart+1)
  double *Z = V + n * (restart + 1);         // n x restart
  double *w = Z + n * restart;               // n
  double *hcol = w + n;                      // restart+1 (device)
  std::vector<double> H((restart + 1) * restart, 0.0), cs(restart), sn(restart), g(restart + 1);
  std::vector<double> hh(restart + 1), est(restart);
  constexpr int STALL_WINDOW = 16;
  GB_CUDA(cudaMemsetAsync(d, 0, n * sizeof(double), s));
  // initial residual of the correction equation: r - A*0 = r
  double beta = 0.0, prev_beta = 0.0;
  GB_CUDA(cudaMemcpyAsync(w, r, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  int total = 0;
  for (int outer = 0; total < max_it; ++outer) {
    // beta = ||w||
    { multidot_kernel<<<1, 256, 0, s>>>(n, w, n, w, hcol); count_launch(); }
    GB_CUDA(cudaMemcpyAsync(M.hx->p, hcol, sizeof(double), cudaMemcpyDeviceToHost, s));
    int st = finish_blocking(s);
    if (st) return st;
    beta = sqrt(M.hx->p[0]);
    if (config().verbose >= 2)
      fprintf(stderr, "libgbblas fgmres: restart %d  ||r|| = %.3e after %d iterations\n", outer,
              beta, total);
    if (outer == 0) rtol *= beta;
    if (beta <= rtol || beta == 0.0) break;
    // a full restart cycle that did not reduce the residual a hundredfold:
    // GMRES cannot finish within the budget at this rate
    if (outer > 0 && beta > 1e-2 * prev_beta) {
      *hopeless = true;
      break;
    }
    prev_beta = beta;
    { scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, 1.0 / beta, w, V, 0); count_launch(); }
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < restart && total < max_it; ++j, ++total) {
      // z_j = M^-1 v_j ; w = A z_j
      GB_CUDA(cudaMemcpyAsync(Z + j * n, V + j * n, n * sizeof(double), cudaMemcpyDeviceToDevice,
                              s));
      if ((st = M.precond64(Z + j * n))) return st;
      M.gemv_dd(Z + j * n, 1.0, w, 0.0, w);
      // classical Gram-Schmidt, twice (CGS2)
      for (int pass = 0; pass < 2; ++pass) {
        { multidot_kernel<<<(unsigned)(j + 1), 256, 0, s>>>(n, V, n, w, hcol); count_launch(); }
        { multiaxpy_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, j + 1, V, n, hcol, w); count_launch(); }
        GB_CUDA(cudaMemcpyAsync(M.hx->p, hcol, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                                s));
        if ((st = finish_blocking(s))) return st;
        for (int i = 0; i <= j; ++i) hh[i] = (pass == 0 ? 0.0 : hh[i]) + M.hx->p[i];
      }
      { multidot_kernel<<<1, 256, 0, s>>>(n, w, n, w, hcol); count_launch(); }
      GB_CUDA(cudaMemcpyAsync(M.hx->p, hcol, sizeof(double), cudaMemcpyDeviceToHost, s));
      if ((st = finish_blocking(s))) return st;
      const double hnext = sqrt(M.hx->p[0]);
      if (hnext > 0.0) {
        { scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, 1.0 / hnext, w, V + (j + 1) * n, 0); count_launch(); }
      }
      // Givens rotations on the Hessenberg column
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * hh[i] + sn[i] * hh[i + 1];
        hh[i + 1] = -sn[i] * hh[i] + cs[i] * hh[i + 1];
        hh[i] = t;
      }
      double a = hh[j], b = hnext;
      double rr = hypot(a, b);
      cs[j] = rr > 0 ? a / rr : 1.0;
      sn[j] = rr > 0 ? b / rr : 0.0;
      hh[j] = rr;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int i = 0; i <= j; ++i) H[i + j * (restart + 1)] = hh[i];
      est[j] = fabs(g[j + 1]);  // the residual norm of the cycle's iterate
      if (config().verbose >= 3)
        fprintf(stderr, "libgbblas fgmres: iteration %d  ||r|| ~ %.3e\n", total + 1, est[j]);
      if (est[j] <= rtol || hnext == 0.0) {
        ++j;
        ++total;
        break;
      }
      // 16 iterations into the first cycle without a tenfold reduction: the
      // preconditioner leaves too much of the spectrum spread for GMRES to
      // finish (a few outlying directions are resolved by then)
      if (outer == 0 && j + 1 == 16 && est[j] > 0.1 * beta) {
        *hopeless = true;
        ++j;
        ++total;
        break;
      }
      // a stall: 16 iterations that did not halve the residual
      if (j >= STALL_WINDOW && est[j] > 0.5 * est[j - STALL_WINDOW]) {
        *hopeless = true;
        ++j;
        ++total;
        break;
      }
    }
    // y = H \ g ; d += Z y
    std::vector<double> y(j);
    for (int i = j - 1; i >= 0; --i) {
      double t = g[i];
      for (int k = i + 1; k < j; ++k) t -= H[i + k * (restart + 1)] * y[k];
      y[i] = t / H[i + i * (restart + 1)];
    }
    for (int i = 0; i < j; ++i)
      { scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, y[i], Z + i * n, d, 1); count_launch(); }
    if (fabs(g[j]) <= rtol) break;
    if (*hopeless) break;  // d keeps the cycle's best iterate; no further restart
    // new residual of the correction equation: w = r - A d
    M.gemv_dd(d, -1.0, r, 1.0, w);
  }
  *iters = total;
  return check_cuda(cudaGetLastError(), "fgmres");
}

}  // namespace

// Device-pointer mixed solve.  A is overwritten only by the FP64 fallback
// (dsgesv.f:410), as in the reference.
int dsgesv_device(int64_t n, int64_t nrhs, double *A, int64_t lda, int *ipiv, const double *B,
                  int64_t ldb, double *X, int64_t ldx, int *iter, int *info, bool use_gmres,
                  cudaStream_t s) {
  *iter = 0;
  *info = 0;
  if (n == 0) return GB_SUCCESS;
  const int itermax = 30;
  Mixed M;
  M.n = n;
  M.nrhs = nrhs;
  M.A = A;
  M.lda = lda;
  M.B = B;
  M.ldb = ldb;
  M.X = X;
  M.ldx = ldx;
  M.ipiv = ipiv;
  M.s = s;
  M.nchunks = (int)((n + GEMV_COL_CHUNK - 1) / GEMV_COL_CHUNK);
  const size_t bytes_sa = ((size_t)n * n * 4 + 255) & ~size_t(255);
  const size_t bytes_sx = ((size_t)n * nrhs * 4 + 255) & ~size_t(255);
  const size_t bytes_r = ((size_t)n * nrhs * 8 + 255) & ~size_t(255);
  const size_t bytes_p = ((size_t)n * (M.nchunks > 64 ? M.nchunks : 64) * 8 + 255) & ~size_t(255);
  const int64_t nblk64 = (n + 63) / 64;
  const size_t bytes_inv = ((size_t)nblk64 * 64 * 64 * 4 + 255) & ~size_t(255);
  const size_t bytes_perm = ((size_t)n * 4 + 255) & ~size_t(255);
  Scratch ws2(bytes_sx + 2 * bytes_inv + bytes_perm, s);
  if (!ws2.p) return GB_ERR_ALLOC;
  M.SX2 = ws2.as<float>();
  M.Linv = reinterpret_cast<float *>(ws2.as<char>() + bytes_sx);
  M.Uinv = reinterpret_cast<float *>(ws2.as<char>() + bytes_sx + bytes_inv);
  M.perm = reinterpret_cast<int *>(ws2.as<char>() + bytes_sx + 2 * bytes_inv);
  Scratch ws(bytes_sa + bytes_sx + bytes_r + bytes_p + 1024 + (size_t)nrhs * 32, s);
  if (!ws.p) return GB_ERR_ALLOC;
  char *base = ws.as<char>();
  M.SA = reinterpret_cast<float *>(base);
  M.SX = reinterpret_cast<float *>(base + bytes_sa);
  M.R = reinterpret_cast<double *>(base + bytes_sa + bytes_sx);
  M.part = reinterpret_cast<double *>(base + bytes_sa + bytes_sx + bytes_r);
  M.dnorm = reinterpret_cast<double *>(base + bytes_sa + bytes_sx + bytes_r + bytes_p);
  M.dflag = reinterpret_cast<int *>(M.dnorm + 2 * nrhs + 8);
  // pinned host scratch: column norms (2*nrhs) and GMRES Hessenberg columns (<= 102)
  Host hx((size_t)(2 * nrhs > 128 ? 2 * nrhs : 128) + 64);
  if (!hx.p) return set_error(GB_ERR_ALLOC, "pinned host scratch");
  M.hx = &hx;
  int st;
  bool fallback = false;

  // anrm = ||A||_inf, cte = anrm * eps * sqrt(n) * BWDMAX (dsgesv.f:279-281)
  {
    dim3 g((unsigned)((n + 255) / 256), (unsigned)M.nchunks);
    { absrowsum_kernel<<<g, 256, 0, s>>>(n, n, A, lda, GEMV_COL_CHUNK, M.part); count_launch(); }
    { rowsum_max_kernel<<<1, 256, 0, s>>>(n, M.nchunks, M.part, M.dnorm); count_launch(); }
  }
  GB_CUDA(cudaMemcpyAsync(hx.p, M.dnorm, sizeof(double), cudaMemcpyDeviceToHost, s));
  if ((st = finish_blocking(s))) return st;
  const double anrm = hx.p[0];
  const double cte = anrm * (DBL_EPSILON * 0.5) * sqrt((double)n) * 1.0;

  // SX = fp32(B), SA = fp32(A) with overflow checks (dsgesv.f:291-304)
  GB_CUDA(cudaMemsetAsync(M.dflag, 0, 2 * sizeof(int), s));
  { lag2s_kernel<<<grid_for(n * nrhs), 256, 0, s>>>(n, nrhs, B, ldb, M.SX, n, M.dflag); count_launch(); }
  { lag2s_kernel<<<grid_for(n * n), 256, 0, s>>>(n, n, A, lda, M.SA, n, M.dflag + 1); count_launch(); }
  int *dinfo = M.dflag + 2;
  GB_CUDA(cudaMemcpyAsync(hx.p, M.dflag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  if ((st = finish_blocking(s))) return st;
  int flags[2];
  memcpy(flags, hx.p, sizeof(flags));
  if (flags[0] || flags[1]) {
    *iter = -2;
    fallback = true;
  }
  if (!fallback) {
    // sgetrf (dsgesv.f:310): a singular FP32 factor sends the solve to FP64
    {
      ProfileScope prof("mixed_sgetrf", s);
      if ((st = getrf_device<float>(n, n, M.SA, n, ipiv, dinfo, s))) return st;
    }
    GB_CUDA(cudaMemcpyAsync(hx.p, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    if ((st = finish_blocking(s))) return st;
    int sinfo;
    memcpy(&sinfo, hx.p, sizeof(int));
    if (sinfo != 0) {
      *iter = -3;
      fallback = true;
    }
  }
  if (!fallback) {
    // once per factorisation: the final permutation and the inverted diagonal blocks
    if ((st = pivots_to_perm(n, ipiv, M.perm, s))) return st;
    if ((st = lu_block_inverses<float>(n, M.SA, n, M.Linv, M.Uinv, s))) return st;
    {
      ProfileScope prof("mixed_getrs", s);
      if ((st = M.solve32(M.SX, nrhs))) return st;
    }
    { lag2d_kernel<<<grid_for(n * nrhs), 256, 0, s>>>(n, nrhs, M.SX, n, X, ldx, 0); count_launch(); }
    double prev = INFINITY, best = INFINITY;
    int stalls = 0;
    bool done = false;
    Scratch xbest(use_gmres ? (size_t)n * nrhs * sizeof(double) : 0, s);
    for (int it = 0; it <= itermax; ++it) {
      if ((st = M.residual())) return st;
      bool ok = false;
      double worst = 0.0;
      if ((st = M.converged(cte, &ok, &worst))) return st;
      if (config().verbose >= 2)
        fprintf(stderr, "libgbblas dsgesv: refinement %d  max|r|/max|x| = %.3e (cte %.3e)\n", it,
                worst, cte);
      if (ok) {
        *iter = it;
        done = true;
        break;
      }
      if (it == itermax) break;
      if (use_gmres) {
        // refinement that diverges or stops contracting hands the best
        // iterate so far over to GMRES-IR
        if (!(worst < 2.0 * best)) {
          GB_CUDA(cudaMemcpy2DAsync(X, ldx * 8, xbest.p, n * 8, n * 8, nrhs,
                                    cudaMemcpyDeviceToDevice, s));
          break;
        }
        if (worst < best) {
          best = worst;
          GB_CUDA(cudaMemcpy2DAsync(xbest.p, n * 8, X, ldx * 8, n * 8, nrhs,
                                    cudaMemcpyDeviceToDevice, s));
        }
        stalls = (worst > 0.5 * prev) ? stalls + 1 : 0;
        prev = worst;
        if (it >= 1 && stalls >= 2) break;
      }
      bool ovf = false;
      if ((st = M.precond(M.R, n, nrhs, &ovf))) return st;
      if (ovf) {
        *iter = -2;
        fallback = true;
        break;
      }
      { lag2d_kernel<<<grid_for(n * nrhs), 256, 0, s>>>(n, nrhs, M.SX, n, X, ldx, 1); count_launch(); }
    }
    if (!done && !fallback && use_gmres) {
      // GMRES-IR: x += FGMRES(A, r) per column until the dsgesv test passes
      Scratch lu64((size_t)n * n * sizeof(double), s);
      if (!lu64.p) return GB_ERR_ALLOC;
      M.LU64 = lu64.as<double>();
      { lag2d_kernel<<<grid_for(n * n), 256, 0, s>>>(n, n, M.SA, n, M.LU64, n, 0); count_launch(); }
      const int64_t nblk64 = (n + 63) / 64;
      Scratch gm_ws(((size_t)2 * nblk64 * 64 * 64 + (size_t)n + (size_t)M.nchunks * n) *
                        sizeof(double), s);
      if (!gm_ws.p) return GB_ERR_ALLOC;
      M.Linv64 = gm_ws.as<double>();
      M.Uinv64 = M.Linv64 + nblk64 * 64 * 64;
      M.W64 = M.Uinv64 + nblk64 * 64 * 64;
      M.part_lo = M.W64 + n;
      if ((st = lu_block_inverses<double>(n, M.LU64, n, M.Linv64, M.Uinv64, s))) return st;
      double prev_worst = INFINITY;
      int total_gm = 0;
      const int gm_restart = n < 48 ? (int)n : 48;  // Hessenberg column fits the host scratch
      const int gm_max = n < 400 ? (int)n : 400;
      bool hopeless = false;
      for (int outer = 0; outer < 4 && !done && !hopeless; ++outer) {
        if ((st = M.residual())) return st;
        bool ok = false;
        double worst = 0.0;
        if ((st = M.converged(cte, &ok, &worst))) return st;
        if (ok) {
          done = true;
          break;
        }
        if (worst > 0.5 * prev_worst) break;  // an outer step that gained nothing: FP64 LU
        prev_worst = worst;
        Scratch dbuf((size_t)n * sizeof(double), s);
        if (!dbuf.p) return GB_ERR_ALLOC;
        if (config().verbose >= 2)
          fprintf(stderr, "libgbblas dsgesv: GMRES-IR outer %d  max|r|/max|x| = %.3e\n", outer,
                  worst);
        for (int64_t j = 0; j < nrhs; ++j) {
          int gi = 0;
          bool hj = false;
          if ((st = fgmres(M, M.R + j * n, dbuf.as<double>(), gm_restart, gm_max, 1e-14, &gi,
                           &hj)))
            return st;
          total_gm += gi;
          if (hj) {  // this column cannot converge: straight to the FP64-accurate LU
            hopeless = true;
            break;
          }
          { scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, 1.0, dbuf.as<double>(), X + j * ldx, 1); count_launch(); }
        }
      }
      if (done) *iter = 100 + total_gm;
    }
    if (!done && !fallback) {
      *iter = -itermax - 1;
      fallback = true;
    }
  }
  if (fallback) {
    // dsgesv.f:410-425: FP64 LU of A (overwritten) and solve
    const int mode = (use_gmres || gb_get_dgemm_mode() != GB_DGEMM_NATIVE) ? 1 : 0;
    if ((st = getrf_device_mode<double>(n, n, A, lda, ipiv, dinfo, mode, s))) return st;
    GB_CUDA(cudaMemcpyAsync(hx.p, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    if ((st = finish_blocking(s))) return st;
    int dinf;
    memcpy(&dinf, hx.p, sizeof(int));
    if (dinf != 0) {
      *info = dinf;
      return GB_SUCCESS;
    }
    GB_CUDA(cudaMemcpy2DAsync(X, ldx * 8, B, ldb * 8, n * 8, nrhs, cudaMemcpyDeviceToDevice, s));
    if ((st = getrs_device<double>(0, n, nrhs, A, lda, ipiv, X, ldx, s))) return st;
  }
  return finish_blocking(s);
}

// Mixed-precision Cholesky solve, lapack-netlib/SRC/dsposv.f:232-434: the
// reference's steps and ITER codes (-2 FP32 overflow, -3 SPOTRF failure,
// -31 no convergence in ITERMAX=30 steps) with the FP32 factorisation and
// solves on the GPU.  The symmetric products (DLANSY, DSYMM) use one full
// FP64 copy of A mirrored from its stored triangle; the FP32 factor is
// mirrored onto its other half so the chained two-triangle solve applies
// (L then L^T, or U^T then U).  A is overwritten only by the FP64 fallback
// (dsposv.f:425-433: DPOTRF, DPOTRS).
int dsposv_device(int uplo, int64_t n, int64_t nrhs, double *A, int64_t lda, const double *B,
                  int64_t ldb, double *X, int64_t ldx, int *iter, int *info, cudaStream_t s) {
  *iter = 0;
  *info = 0;
  if (n == 0) return GB_SUCCESS;
  const int itermax = 30;
  const int lower = uplo == 1;
  Scratch full((size_t)n * n * sizeof(double), s);
  if (!full.p) return GB_ERR_ALLOC;
  double *Af = full.as<double>();
  GB_CUDA(cudaMemcpy2DAsync(Af, n * 8, A, lda * 8, n * 8, n, cudaMemcpyDeviceToDevice, s));
  int st = mirror_triangle<double>(n, Af, n, lower, s);
  if (st) return st;
  Mixed M;
  M.chol = true;
  M.n = n;
  M.nrhs = nrhs;
  M.A = Af;
  M.lda = n;
  M.B = B;
  M.ldb = ldb;
  M.X = X;
  M.ldx = ldx;
  M.s = s;
  M.nchunks = (int)((n + GEMV_COL_CHUNK - 1) / GEMV_COL_CHUNK);
  const size_t bytes_sa = ((size_t)n * n * 4 + 255) & ~size_t(255);
  const size_t bytes_sx = ((size_t)n * nrhs * 4 + 255) & ~size_t(255);
  const size_t bytes_r = ((size_t)n * nrhs * 8 + 255) & ~size_t(255);
  const size_t bytes_p = ((size_t)n * (M.nchunks > 64 ? M.nchunks : 64) * 8 + 255) & ~size_t(255);
  const int64_t nblk64 = (n + 63) / 64;
  const size_t bytes_inv = ((size_t)nblk64 * 64 * 64 * 4 + 255) & ~size_t(255);
  Scratch ws2(bytes_sx + 2 * bytes_inv, s);
  if (!ws2.p) return GB_ERR_ALLOC;
  M.SX2 = ws2.as<float>();
  M.Linv = reinterpret_cast<float *>(ws2.as<char>() + bytes_sx);
  M.Uinv = reinterpret_cast<float *>(ws2.as<char>() + bytes_sx + bytes_inv);
  Scratch ws(bytes_sa + bytes_sx + bytes_r + bytes_p + 1024 + (size_t)nrhs * 32, s);
  if (!ws.p) return GB_ERR_ALLOC;
  char *base = ws.as<char>();
  M.SA = reinterpret_cast<float *>(base);
  M.SX = reinterpret_cast<float *>(base + bytes_sa);
  M.R = reinterpret_cast<double *>(base + bytes_sa + bytes_sx);
  M.part = reinterpret_cast<double *>(base + bytes_sa + bytes_sx + bytes_r);
  M.dnorm = reinterpret_cast<double *>(base + bytes_sa + bytes_sx + bytes_r + bytes_p);
  M.dflag = reinterpret_cast<int *>(M.dnorm + 2 * nrhs + 8);
  Host hx((size_t)(2 * nrhs > 128 ? 2 * nrhs : 128) + 64);
  if (!hx.p) return set_error(GB_ERR_ALLOC, "pinned host scratch");
  M.hx = &hx;
  bool fallback = false;

  // anrm = DLANSY('I') = ||A||_inf of the symmetric matrix (dsposv.f:282-284)
  {
    dim3 g((unsigned)((n + 255) / 256), (unsigned)M.nchunks);
    { absrowsum_kernel<<<g, 256, 0, s>>>(n, n, Af, n, GEMV_COL_CHUNK, M.part); count_launch(); }
    { rowsum_max_kernel<<<1, 256, 0, s>>>(n, M.nchunks, M.part, M.dnorm); count_launch(); }
  }
  GB_CUDA(cudaMemcpyAsync(hx.p, M.dnorm, sizeof(double), cudaMemcpyDeviceToHost, s));
  if ((st = finish_blocking(s))) return st;
  const double cte = hx.p[0] * (DBL_EPSILON * 0.5) * sqrt((double)n) * 1.0;

  // SX = fp32(B), SA = fp32(A) with overflow checks (dsposv.f:291-304; the
  // mirrored copy holds exactly the stored triangle's values)
  GB_CUDA(cudaMemsetAsync(M.dflag, 0, 3 * sizeof(int), s));
  { lag2s_kernel<<<grid_for(n * nrhs), 256, 0, s>>>(n, nrhs, B, ldb, M.SX, n, M.dflag); count_launch(); }
  { lag2s_kernel<<<grid_for(n * n), 256, 0, s>>>(n, n, Af, n, M.SA, n, M.dflag + 1); count_launch(); }
  int *dinfo = M.dflag + 2;
  GB_CUDA(cudaMemcpyAsync(hx.p, M.dflag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  if ((st = finish_blocking(s))) return st;
  int flags[2];
  memcpy(flags, hx.p, sizeof(flags));
  if (flags[0] || flags[1]) {
    *iter = -2;
    fallback = true;
  }
  if (!fallback) {
    // spotrf (dsposv.f:310): a failed FP32 factor sends the solve to FP64
    {
      ProfileScope prof("mixed_spotrf", s);
      if ((st = spotrf_device(uplo, n, M.SA, n, dinfo, s))) return st;
    }
    GB_CUDA(cudaMemcpyAsync(hx.p, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    if ((st = finish_blocking(s))) return st;
    int sinfo;
    memcpy(&sinfo, hx.p, sizeof(int));
    if (sinfo != 0) {
      *iter = -3;
      fallback = true;
    }
  }
  if (!fallback) {
    if ((st = mirror_triangle<float>(n, M.SA, n, lower, s))) return st;
    if ((st = chol_block_inverses<float>(n, M.SA, n, M.Linv, M.Uinv, s))) return st;
    if ((st = M.solve32(M.SX, nrhs))) return st;
    { lag2d_kernel<<<grid_for(n * nrhs), 256, 0, s>>>(n, nrhs, M.SX, n, X, ldx, 0); count_launch(); }
    bool done = false;
    for (int it = 0; it <= itermax; ++it) {
      if ((st = M.residual())) return st;
      bool ok = false;
      double worst = 0.0;
      if ((st = M.converged(cte, &ok, &worst))) return st;
      if (config().verbose >= 2)
        fprintf(stderr, "libgbblas dsposv: refinement %d  max|r|/max|x| = %.3e (cte %.3e)\n", it,
                worst, cte);
      if (ok) {
        *iter = it;
        done = true;
        break;
      }
      if (it == itermax) break;
      bool ovf = false;
      if ((st = M.precond(M.R, n, nrhs, &ovf))) return st;
      if (ovf) {
        *iter = -2;
        fallback = true;
        break;
      }
      { lag2d_kernel<<<grid_for(n * nrhs), 256, 0, s>>>(n, nrhs, M.SX, n, X, ldx, 1); count_launch(); }
    }
    if (!done && !fallback) {
      *iter = -itermax - 1;
      fallback = true;
    }
  }
  if (fallback) {
    const int mode = gb_get_dgemm_mode() != GB_DGEMM_NATIVE ? 1 : 0;
    if ((st = potrf_device(uplo, n, A, lda, dinfo, mode, s))) return st;
    GB_CUDA(cudaMemcpyAsync(hx.p, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s));
    if ((st = finish_blocking(s))) return st;
    int dinf;
    memcpy(&dinf, hx.p, sizeof(int));
    if (dinf != 0) {
      *info = dinf;
      return GB_SUCCESS;
    }
    GB_CUDA(cudaMemcpy2DAsync(X, ldx * 8, B, ldb * 8, n * 8, nrhs, cudaMemcpyDeviceToDevice, s));
    if ((st = potrs_device(uplo, n, nrhs, A, lda, X, ldx, s))) return st;
  }
  return finish_blocking(s);
}

}  // namespace gb

using namespace gb;

extern "C" {

int dsgesv_(const blasint *N, const blasint *NRHS, double *a, const blasint *ldA, blasint *ipiv,
            const double *b, const blasint *ldB, double *x, const blasint *ldX, double *work,
            float *swork, blasint *ITER, blasint *Info) {
  (void)work;
  (void)swork;
  int64_t n = *N, nrhs = *NRHS, lda = *ldA, ldb = *ldB, ldx = *ldX;
  *ITER = 0;
  int info = 0;
  // dsgesv.f:236-249 (argument checks, XERBLA with the positive position)
  if (n < 0) info = 1;
  else if (nrhs < 0) info = 2;
  else if (lda < (n > 1 ? n : 1)) info = 4;
  else if (ldb < (n > 1 ? n : 1)) info = 7;
  else if (ldx < (n > 1 ? n : 1)) info = 9;
  if (info) {
    *Info = -info;
    call_xerbla("DSGESV", info);
    return 0;
  }
  *Info = 0;
  if (n == 0) return 0;
  if (ensure_init()) return 0;
  cudaStream_t s = stream();
  Operand A(a, n, n, lda, 8), B(b, n, nrhs, ldb, 8), X(x, n, nrhs, ldx, 8);
  if (A.bind(true, s) || B.bind(true, s) || X.bind(false, s)) return 0;
  Scratch piv((size_t)n * sizeof(int), s);
  int *dpiv = is_device_pointer(ipiv) ? ipiv : piv.as<int>();
  int it = 0, inf = 0;
  // the Fortran entry keeps the reference's behaviour (no GMRES stage)
  if (dsgesv_device(n, nrhs, A.d<double>(), A.dld, dpiv, B.d<double>(), B.dld, X.d<double>(),
                    X.dld, &it, &inf, false, s))
    return 0;
  if (it < 0) A.unbind(s);  // A holds the FP64 LU only after a fallback
  X.unbind(s);
  if (dpiv != ipiv) cudaMemcpyAsync(ipiv, dpiv, n * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (finish_blocking(s)) return 0;
  *ITER = it;
  *Info = inf;
  return 0;
}

int gb_dsgesv_dev(int64_t n, int64_t nrhs, double *A, int64_t lda, int *ipiv, const double *B,
                  int64_t ldb, double *X, int64_t ldx, int *iter, int *info) {
  int code = 0;
  if (n < 0) code = 1;
  else if (nrhs < 0) code = 2;
  else if (lda < (n > 1 ? n : 1)) code = 4;
  else if (ldb < (n > 1 ? n : 1)) code = 7;
  else if (ldx < (n > 1 ? n : 1)) code = 9;
  if (code) {
    call_xerbla("DSGESV", code);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  return dsgesv_device(n, nrhs, A, lda, ipiv, B, ldb, X, ldx, iter, info, true, stream());
}

// dsposv.f:236-251: checks in order UPLO, N, NRHS, LDA, LDB, LDX
static int dsposv_checks(char u, int64_t n, int64_t nrhs, int64_t lda, int64_t ldb, int64_t ldx,
                         int *uplo) {
  *uplo = u == 'U' ? 0 : u == 'L' ? 1 : -1;
  if (*uplo < 0) return 1;
  if (n < 0) return 2;
  if (nrhs < 0) return 3;
  if (lda < (n > 1 ? n : 1)) return 5;
  if (ldb < (n > 1 ? n : 1)) return 7;
  if (ldx < (n > 1 ? n : 1)) return 9;
  return 0;
}

int dsposv_(const char *UPLO, const blasint *N, const blasint *NRHS, double *a,
            const blasint *ldA, const double *b, const blasint *ldB, double *x,
            const blasint *ldX, double *work, float *swork, blasint *ITER, blasint *Info) {
  (void)work;
  (void)swork;
  int64_t n = *N, nrhs = *NRHS, lda = *ldA, ldb = *ldB, ldx = *ldX;
  *ITER = 0;
  int uplo = 0;
  const int code = dsposv_checks(upch(UPLO), n, nrhs, lda, ldb, ldx, &uplo);
  if (code) {
    *Info = -code;
    call_xerbla("DSPOSV", code);
    return 0;
  }
  *Info = 0;
  if (n == 0) return 0;
  if (ensure_init()) return 0;
  cudaStream_t s = stream();
  Operand A(a, n, n, lda, 8), B(b, n, nrhs, ldb, 8), X(x, n, nrhs, ldx, 8);
  if (A.bind(true, s) || B.bind(true, s) || X.bind(false, s)) return 0;
  int it = 0, inf = 0;
  if (dsposv_device(uplo, n, nrhs, A.d<double>(), A.dld, B.d<double>(), B.dld, X.d<double>(),
                    X.dld, &it, &inf, s))
    return 0;
  if (it < 0) A.unbind(s);  // A holds the FP64 factor only after a fallback
  X.unbind(s);
  if (finish_blocking(s)) return 0;
  *ITER = it;
  *Info = inf;
  return 0;
}

int gb_dsposv_dev(char uplo, int64_t n, int64_t nrhs, double *A, int64_t lda, const double *B,
                  int64_t ldb, double *X, int64_t ldx, int *iter, int *info) {
  int up = 0;
  const int code = dsposv_checks(upch(uplo), n, nrhs, lda, ldb, ldx, &up);
  if (code) {
    call_xerbla("DSPOSV", code);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  return dsposv_device(up, n, nrhs, A, lda, B, ldb, X, ldx, iter, info, stream());
}

}  // extern "C"
