// LU solve with inverted diagonal blocks, one launch per triangle.
//
// getrs (lapack/getrs/getrs_single.c:42-68) applies the interchanges and two
// triangular solves; for one right-hand side the reference switches to TRSV
// (driver/level2/trsv_L.c, trsv_U.c), a latency-bound sweep.  Here the
// diagonal blocks (TB x TB) of the unit-lower L and of U are inverted once
// per factorisation.  A solve is then one kernel per triangle in which each
// CTA owns one 64-row block of the solution for a group of right-hand
// sides: it takes a ticket from an atomic counter (block order = ticket
// order, so every block it waits for belongs to a CTA that is already
// running), accumulates A(i, j) x_j over the finished blocks j as their
// release flags appear, and finishes with x_i = inv(D_ii) (b_i - sum).  The
// triangle is read once, by all CTAs in parallel; only the short dependency
// tail of each block is serial.  Every wait is bounded: on timeout the
// kernel records GB_KERR_CHAIN_TIMEOUT in the status word and returns.
// Used by the mixed-precision solver's refinement steps, where the factors
// are reused many times.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_internal.h"
#include "lapack_internal.h"

namespace gb {

namespace {

constexpr int TB = 64;           // diagonal block size
// right-hand sides per chain (accumulators per thread)
template <typename T>
constexpr int maxr() { return sizeof(T) == 4 ? 8 : 4; }

// Inverse of a diagonal block of the lower (lower = 1) or upper (lower = 0)
// triangle, unit diagonal when `unit` (the L of an LU) and non-unit
// otherwise.  One CTA per block, thread c computes column c of the inverse
// by substitution on e_c.  Blocks shorter than TB are padded with identity.
template <typename T>
__global__ void __launch_bounds__(TB)
diag_inverse_kernel(int64_t n, const T *__restrict__ A, int64_t lda, int lower, int unit,
                    T *__restrict__ inv) {
  __shared__ T D[TB][TB + 1];
  const int64_t b = blockIdx.x;
  const int64_t r0 = b * TB;
  const int nb = (int)((n - r0) < TB ? (n - r0) : TB);
  for (int e = threadIdx.x; e < TB * TB; e += TB) {
    const int r = e % TB, c = e / TB;
    T v = T(0);
    if (r < nb && c < nb) v = A[(r0 + r) + (r0 + c) * lda];
    if (r == c && (r >= nb || unit)) v = T(1);  // unit diagonal, identity padding
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
      x[r] = unit ? s : s / D[r][r];
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

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr uint64_t CHAIN_WAIT_NS = 2000000000ull;

// One triangle of the solve.  lower = 1: L y = b (blocks in ascending
// order, inverses of L); lower = 0: U x = y (descending, inverses of U).
// Bin is read only; Xout receives the solution blocks, which other CTAs of
// the same launch read back (through L2) once the block's flag is set.
// flags[grp * nblk + i] = 1 when block i of right-hand-side group grp is
// final.  Thread (r, g4) owns row r of the block and columns g4*16..+16 of
// each 64-column tile of A; U tiles are in flight per step.
template <typename T, int R, int U>
__global__ void __launch_bounds__(256)
chain_solve_kernel(int64_t n, int nrhs, const T *__restrict__ A, int64_t lda,
                   const T *__restrict__ inv, int lower, const T *__restrict__ Bin, int64_t ldb,
                   T *Xout, int64_t ldx, int *flags, int *ticket, int nblk, int ngroups,
                   int *status) {
  __shared__ T xs[U][R][TB];
  __shared__ T red[4][R][TB];
  __shared__ int s_val;
  const int tid = threadIdx.x, r = tid & (TB - 1), g4 = tid >> 6;
  if (tid == 0) s_val = atomicAdd(ticket, 1);
  __syncthreads();
  const int t = s_val;
  const int idx = t / ngroups, grp = t - idx * ngroups;
  const int i = lower ? idx : nblk - 1 - idx;
  const int64_t r0 = (int64_t)i * TB;
  const int nb = (int)((n - r0) < TB ? (n - r0) : TB);
  const int k0 = grp * R;
  const int kk = (nrhs - k0) < R ? (nrhs - k0) : R;
  int *fl = flags + (int64_t)grp * nblk;
  auto chain = [&](int jj) { return lower ? jj : nblk - 1 - jj; };

  T iv[16];
  {
    const T *ivb = inv + (int64_t)i * (TB * TB);
#pragma unroll
    for (int c = 0; c < 16; ++c) iv[c] = ivb[r + (g4 * 16 + c) * TB];
  }
  T acc[R];
#pragma unroll
  for (int k = 0; k < R; ++k) acc[k] = T(0);
  const T *Arow = A + r0 + r;
  const bool row_ok = r < nb;

  int ready = -1;  // dependencies 0..ready (in chain order) are final
  int jj = 0;
  while (jj < idx) {
    const int jmax = (idx - jj) < U ? (idx - jj) : U;
    // the A tiles do not depend on the solution: issue them before waiting
    T a[U][16];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (u < jmax) {
        const int64_t c0 = (int64_t)chain(jj + u) * TB + g4 * 16;
#pragma unroll
        for (int c = 0; c < 16; ++c)
          a[u][c] = (row_ok && c0 + c < n) ? Arow[(c0 + c) * lda] : T(0);
      }
    }
    if (jj > ready) {
      __syncthreads();  // every thread has read s_val
      if (tid == 0) {
        int rd = -2;
        if (ld_acquire(&fl[chain(idx - 1)])) {
          rd = idx - 1;  // a flag implies all earlier flags of the chain
        } else {
          const uint64_t t0 = now_ns();
          for (;;) {
            if (ld_acquire(&fl[chain(jj)])) {
              rd = jj;
              break;
            }
            if (*(volatile int *)status) break;  // another block gave up
            if (now_ns() - t0 > CHAIN_WAIT_NS) {
              atomicCAS(status, 0, GB_KERR_CHAIN_TIMEOUT);
              atomicExch(status + 1, 100 + lower);
              break;
            }
            __nanosleep(100);
          }
          if (rd >= 0)
            while (rd + 1 < idx && rd + 1 < jj + U && ld_acquire(&fl[chain(rd + 1)])) ++rd;
        }
        s_val = rd;
      }
      __syncthreads();
      ready = s_val;
      if (ready < 0) return;  // uniform: every thread read the same value
    }
    const int jn = (ready - jj + 1) < jmax ? (ready - jj + 1) : jmax;
    for (int e = tid; e < jn * R * TB; e += 256) {
      const int u = e / (R * TB), k = (e / TB) % R, c = e % TB;
      const int64_t col = (int64_t)chain(jj + u) * TB + c;
      xs[u][k][c] = (k < kk && col < n) ? __ldcg(&Xout[col + (int64_t)(k0 + k) * ldx]) : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (u < jn) {
#pragma unroll
        for (int c = 0; c < 16; ++c)
#pragma unroll
          for (int k = 0; k < R; ++k) acc[k] = fma(a[u][c], xs[u][k][g4 * 16 + c], acc[k]);
      }
    }
    __syncthreads();
    jj += jn;
  }

  // v = b_i - sum_j A(i, j) x_j, then x_i = inv(D_ii) v
#pragma unroll
  for (int k = 0; k < R; ++k) red[g4][k][r] = acc[k];
  __syncthreads();
  for (int e = tid; e < R * TB; e += 256) {
    const int k = e / TB, rr = e % TB;
    T v = T(0);
    if (k < kk && rr < nb)
      v = Bin[(r0 + rr) + (int64_t)(k0 + k) * ldb] -
          ((red[0][k][rr] + red[1][k][rr]) + (red[2][k][rr] + red[3][k][rr]));
    xs[0][k][rr] = v;
  }
  __syncthreads();
  T p[R];
#pragma unroll
  for (int k = 0; k < R; ++k) {
    p[k] = T(0);
#pragma unroll
    for (int c = 0; c < 16; ++c) p[k] = fma(iv[c], xs[0][k][g4 * 16 + c], p[k]);
  }
#pragma unroll
  for (int k = 0; k < R; ++k) red[g4][k][r] = p[k];
  __syncthreads();
  for (int e = tid; e < R * TB; e += 256) {
    const int k = e / TB, rr = e % TB;
    if (k < kk && rr < nb)
      Xout[(r0 + rr) + (int64_t)(k0 + k) * ldx] =
          (red[0][k][rr] + red[1][k][rr]) + (red[2][k][rr] + red[3][k][rr]);
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) st_release(&fl[i], 1);
}

}  // namespace

template <typename T>
int lu_block_inverses(int64_t n, const T *A, int64_t lda, T *Linv, T *Uinv, cudaStream_t s) {
  const unsigned nblk = (unsigned)((n + TB - 1) / TB);
  { diag_inverse_kernel<T><<<nblk, TB, 0, s>>>(n, A, lda, 1, 1, Linv); count_launch(); }
  { diag_inverse_kernel<T><<<nblk, TB, 0, s>>>(n, A, lda, 0, 0, Uinv); count_launch(); }
  return check_cuda(cudaGetLastError(), "diag_inverse");
}

// Cholesky: both triangles of the mirrored factor have non-unit diagonals.
template <typename T>
int chol_block_inverses(int64_t n, const T *A, int64_t lda, T *Linv, T *Uinv, cudaStream_t s) {
  const unsigned nblk = (unsigned)((n + TB - 1) / TB);
  { diag_inverse_kernel<T><<<nblk, TB, 0, s>>>(n, A, lda, 1, 0, Linv); count_launch(); }
  { diag_inverse_kernel<T><<<nblk, TB, 0, s>>>(n, A, lda, 0, 0, Uinv); count_launch(); }
  return check_cuda(cudaGetLastError(), "diag_inverse");
}

// Copy the strictly lower triangle onto the strictly upper one, transposed
// (from_lower = 1), or the other way round: a Cholesky factor L (or U) then
// holds L^T (U^T) in its other half, and the two-triangle solve applies.
template <typename T>
__global__ void mirror_triangle_kernel(int64_t n, T *__restrict__ A, int64_t lda, int from_lower) {
  __shared__ T tile[32][33];
  const int64_t bi = blockIdx.y, bj = blockIdx.x;  // source tile (rows bi, cols bj), bi >= bj
  if (bi < bj) return;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  // read the source triangle, coalesced along the rows of the source tile;
  // tile[a][b] always holds the pair (r, c) = (bi*32 + a, bj*32 + b), r > c
  if (from_lower) {
    for (int yy = ty; yy < 32; yy += 8) {
      const int64_t r = bi * 32 + tx, c = bj * 32 + yy;  // lower element (r, c)
      if (r < n && c < n && r > c) tile[tx][yy] = A[r + c * lda];
    }
  } else {
    for (int yy = ty; yy < 32; yy += 8) {
      const int64_t r = bi * 32 + yy, c = bj * 32 + tx;  // upper element (c, r)
      if (r < n && c < n && r > c) tile[yy][tx] = A[c + r * lda];
    }
  }
  __syncthreads();
  if (from_lower) {
    for (int yy = ty; yy < 32; yy += 8) {
      const int64_t r = bi * 32 + yy, c = bj * 32 + tx;  // write (c, r) = (r, c)
      if (r < n && c < n && r > c) A[c + r * lda] = tile[yy][tx];
    }
  } else {
    for (int yy = ty; yy < 32; yy += 8) {
      const int64_t r = bi * 32 + tx, c = bj * 32 + yy;  // write (r, c) = (c, r)
      if (r < n && c < n && r > c) A[r + c * lda] = tile[tx][yy];
    }
  }
}

template <typename T>
int mirror_triangle(int64_t n, T *A, int64_t lda, int from_lower, cudaStream_t s) {
  if (n <= 1) return GB_SUCCESS;
  const unsigned nt = (unsigned)((n + 31) / 32);
  { mirror_triangle_kernel<T><<<dim3(nt, nt), 256, 0, s>>>(n, A, lda, from_lower); count_launch(); }
  return check_cuda(cudaGetLastError(), "mirror_triangle");
}

template <typename T, int R>
static void launch_chain(unsigned grid, int64_t n, int nrhs, const T *A, int64_t lda,
                         const T *inv, int lower, const T *Bin, int64_t ldb, T *Xout, int64_t ldx,
                         int *flags, int *ticket, int nblk, int ngroups, cudaStream_t s) {
  constexpr int U = sizeof(T) == 4 ? 4 : 2;
  chain_solve_kernel<T, R, U><<<grid, 256, 0, s>>>(n, nrhs, A, lda, inv, lower, Bin, ldb, Xout,
                                                   ldx, flags, ticket, nblk, ngroups,
                                                   ctx().d_status);
  count_launch();
}

// Solve L U X = B in place (interchanges already applied): the forward
// triangle reads B and writes y to scratch, the backward triangle reads y
// and writes x back into B.  Right-hand sides are solved in groups of R
// columns, each group an independent chain of blocks.
template <typename T>
int lu_block_solve(int64_t n, int64_t nrhs, const T *A, int64_t lda, const T *Linv,
                   const T *Uinv, T *B, int64_t ldb, cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return GB_SUCCESS;
  const int nblk = (int)((n + TB - 1) / TB);
  const int R = nrhs == 1 ? 1 : (nrhs <= 4 ? 4 : maxr<T>());
  const int ngroups = (int)((nrhs + R - 1) / R);
  const size_t ybytes = (((size_t)n * nrhs * sizeof(T)) + 255) & ~size_t(255);
  const size_t nflags = 2 * (size_t)ngroups * nblk + 2;
  Scratch ws(ybytes + nflags * sizeof(int), s);
  if (!ws.p) return GB_ERR_ALLOC;
  T *Y = ws.as<T>();
  int *flags = reinterpret_cast<int *>(static_cast<char *>(ws.p) + ybytes);
  int *tickets = flags + 2 * (size_t)ngroups * nblk;
  GB_CUDA(cudaMemsetAsync(flags, 0, nflags * sizeof(int), s));
  const unsigned grid = (unsigned)nblk * (unsigned)ngroups;
  const int k = (int)nrhs;
  for (int pass = 0; pass < 2; ++pass) {
    const int lower = pass == 0;
    const T *inv = lower ? Linv : Uinv;
    const T *Bin = lower ? B : Y;
    const int64_t lbin = lower ? ldb : n;
    T *Xo = lower ? Y : B;
    const int64_t lxo = lower ? n : ldb;
    int *fl = flags + (size_t)pass * ngroups * nblk;
    if (R == 1)
      launch_chain<T, 1>(grid, n, k, A, lda, inv, lower, Bin, lbin, Xo, lxo, fl, tickets + pass,
                         nblk, ngroups, s);
    else if (R == 4)
      launch_chain<T, 4>(grid, n, k, A, lda, inv, lower, Bin, lbin, Xo, lxo, fl, tickets + pass,
                         nblk, ngroups, s);
    else
      launch_chain<T, maxr<T>()>(grid, n, k, A, lda, inv, lower, Bin, lbin, Xo, lxo, fl,
                                 tickets + pass, nblk, ngroups, s);
  }
  return check_cuda(cudaGetLastError(), "lu_block_solve");
}

template int lu_block_inverses<float>(int64_t, const float *, int64_t, float *, float *,
                                      cudaStream_t);
template int lu_block_inverses<double>(int64_t, const double *, int64_t, double *, double *,
                                       cudaStream_t);
template int chol_block_inverses<float>(int64_t, const float *, int64_t, float *, float *,
                                        cudaStream_t);
template int chol_block_inverses<double>(int64_t, const double *, int64_t, double *, double *,
                                         cudaStream_t);
template int mirror_triangle<float>(int64_t, float *, int64_t, int, cudaStream_t);
template int mirror_triangle<double>(int64_t, double *, int64_t, int, cudaStream_t);
template int lu_block_solve<float>(int64_t, int64_t, const float *, int64_t, const float *,
                                   const float *, float *, int64_t, cudaStream_t);
template int lu_block_solve<double>(int64_t, int64_t, const double *, int64_t, const double *,
                                    const double *, double *, int64_t, cudaStream_t);

}  // namespace gb
