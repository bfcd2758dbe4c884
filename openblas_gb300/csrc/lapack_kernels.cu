// LU / Cholesky building blocks on the GPU: the partial-pivot panel
// factorisation, row interchanges (LASWP) and the diagonal-block Cholesky.
//
// Panel LU (lapack/getf2/getf2_k.c:46-125 semantics).  The m x nb panel is
// factored by one cooperative launch: every thread owns up to R rows of the
// panel and keeps them in registers for the whole panel.  Per column j:
//   1. each block finds its first-maximum |a_ij| row (IAMAX rule: largest
//      magnitude, smallest index on ties) and publishes the value, the row
//      index and the full row to a parity-buffered slot; the owner of row j
//      also publishes row j;
//   2. one grid barrier;
//   3. every block reduces the candidates to the same pivot p, then each
//      thread updates only its own rows: row j takes the old row p, row p
//      takes the old row j, multipliers l_i = a_ij * (1/pivot) (only when
//      |pivot| >= DBL_MIN, as in getf2_k.c:105-116, where the swap is also
//      skipped), and the rank-1 update a_ic -= l_i * u_c for c > j.
// Because each thread writes only rows it owns and reads the published rows
// from the slot buffers, one barrier per column suffices.  The barrier is a
// bounded spin: if it does not complete within its iteration limit the
// kernel records an error status and returns.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <stdio.h>

#include <cooperative_groups.h>

#include <mutex>

#include "gb_internal.h"
#include "lapack_internal.h"
#include "operand.h"

namespace gb {

namespace {

constexpr int PANEL_THREADS = 256;
constexpr unsigned BARRIER_SPIN_LIMIT = 1u << 24;

// Bounded grid-wide barrier for a cooperatively launched grid.  bar[0] is
// the arrival counter, bar[1] the generation.  Returns false (and sets the
// status word) when the wait limit expires.
__device__ bool grid_barrier(unsigned *bar, unsigned nblocks, int *status, int site) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned *vgen = bar + 1;
    unsigned gen = *vgen;
    __threadfence();
    unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned spins = 0;
      while (*vgen == gen) {
        if (++spins > BARRIER_SPIN_LIMIT) {
          ok = 0;
          atomicCAS(status, 0, GB_KERR_BARRIER_TIMEOUT);
          atomicExch(status + 1, site);
          break;
        }
        if (spins > 64) __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

template <typename T>
__device__ inline T tiny_pivot();
template <>
__device__ inline double tiny_pivot<double>() { return DBL_MIN; }
template <>
__device__ inline float tiny_pivot<float>() { return FLT_MIN; }

// IAMAX of the panel kernels.  getf2_k.c's running maximum starts from
// |a_jj| and only moves to a larger value, so a NaN never becomes the pivot.
// FP32 compares the magnitudes as floats (-1: no candidate).  FP64 compares
// ordered integer keys instead, 0 for NaN and for "no candidate",
// bits(|x|) + 1 otherwise: GB300 has ~2 FP64 operations per clock per SM,
// and the compares of the search and its warp reductions would otherwise
// cost more than the column's rank-1 update.
template <typename T>
struct PivotOps;
template <>
struct PivotOps<float> {
  using V = float;
  __device__ static V none() { return -1.0f; }
  __device__ static V mag(float x) { return x < 0.f ? -x : x; }
  __device__ static bool better(V a, V best, long long row, long long bidx) {
    return a > best || (a == best && row < bidx);
  }
  __device__ static void argmax(V &v, long long &i);  // warp_argmax<float>, below
  __device__ static float carry(V v) { return v; }
  __device__ static V uncarry(float v) { return v; }
  __device__ static bool is_nan(float x) { return x != x; }
  __device__ static bool nonzero(float x) { return x != 0.f; }
  __device__ static bool scaled(float x) { return x != 0.f && (x < 0.f ? -x : x) >= FLT_MIN; }
};
template <>
struct PivotOps<double> {
  using V = unsigned long long;
  __device__ static V none() { return 0ull; }
  __device__ static V mag(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
    return b > 0x7FF0000000000000ull ? 0ull : b + 1ull;
  }
  __device__ static bool better(V a, V best, long long row, long long bidx) {
    return a > best || (a == best && a != 0ull && row < bidx);
  }
  // first maximum over the warp: the largest key, the smallest row among its
  // holders (rows < 2^32 - 1); 0 / LLONG_MAX when no lane has a candidate
  __device__ static void argmax(V &k, long long &i) {
    const unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
    const unsigned hmax = __reduce_max_sync(0xffffffffu, hi);
    const unsigned lmax = __reduce_max_sync(0xffffffffu, hi == hmax ? lo : 0u);
    const unsigned long long kmax = ((unsigned long long)hmax << 32) | lmax;
    const unsigned ik = (k == kmax && kmax != 0ull) ? (unsigned)i : 0xffffffffu;
    const unsigned imin = __reduce_min_sync(0xffffffffu, ik);
    k = kmax;
    i = imin == 0xffffffffu ? LLONG_MAX : (long long)imin;
  }
  __device__ static double carry(V k) { return __longlong_as_double((long long)k); }  // bits
  __device__ static V uncarry(double v) { return (unsigned long long)__double_as_longlong(v); }
  __device__ static bool is_nan(double x) { return mag(x) == 0ull; }
  // piv != 0 (NaN counts) and fabs(piv) >= DBL_MIN (NaN does not), on the key
  __device__ static bool nonzero(double x) { return mag(x) != 1ull; }
  __device__ static bool scaled(double x) { return mag(x) >= mag(DBL_MIN); }
};

// The grid-wide panel's candidate values: FP32 magnitudes (-1: none), FP64
// PivotOps keys carried as the bits of a double (0: none).
template <typename T>
__device__ __forceinline__ T panel_none() {
  if constexpr (sizeof(T) == 4) return T(-1);
  else return PivotOps<double>::carry(PivotOps<double>::none());
}
template <typename T>
__device__ __forceinline__ bool panel_better(T a, T b, int64_t ia, int64_t ib) {
  if constexpr (sizeof(T) == 4) {
    return a > b || (a == b && ia < ib);
  } else {
    const auto ka = PivotOps<double>::uncarry(a), kb = PivotOps<double>::uncarry(b);
    return ka > kb || (ka == kb && ka != 0ull && ia < ib);
  }
}

template <typename T, int R>
__global__ void __launch_bounds__(PANEL_THREADS)
getf2_panel_kernel(int64_t m, int nb, T *__restrict__ A, int64_t lda, int *__restrict__ ipiv,
                   int64_t row_off, int *__restrict__ info, T *__restrict__ slots,
                   unsigned *__restrict__ bar, int *__restrict__ status) {
  // slots layout: [2][nblocks][PANEL_NB + 2] for candidate rows (value, index
  // stored in the two extra entries) + [2][PANEL_NB] for row j.
  const unsigned nblocks = gridDim.x;
  const int64_t nthreads = (int64_t)nblocks * PANEL_THREADS;
  const int64_t gtid = (int64_t)blockIdx.x * PANEL_THREADS + threadIdx.x;
  constexpr int W = PANEL_NB + 2;
  T *cand = slots;                                    // [2][nblocks][W]
  T *rowj_buf = slots + 2 * (int64_t)nblocks * W;     // [2][PANEL_NB]

  T v[R][PANEL_NB];
  int64_t rows[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    rows[r] = gtid + r * nthreads;
#pragma unroll
    for (int c = 0; c < PANEL_NB; ++c)
      v[r][c] = (rows[r] < m && c < nb) ? A[rows[r] + c * lda] : T(0);
  }

  __shared__ T s_val[PANEL_THREADS / 32];
  __shared__ int64_t s_idx[PANEL_THREADS / 32];
  __shared__ int64_t s_best;
  __shared__ T s_u[PANEL_NB];     // new row j (old row p)
  __shared__ T s_oldj[PANEL_NB];  // old row j
  __shared__ int64_t s_p;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = 0; j < nb && j < m; ++j) {
    const int par = j & 1;
    // ---- 1. block-local first-max over rows >= j (FP64: on the integer
    // keys of PivotOps, carried in the T-typed slots as their bits)
    T best = T(-1);
    int64_t bidx = INT64_MAX;
    if constexpr (sizeof(T) == 4) {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (rows[r] < m && rows[r] >= j) {
          T a = v[r][0];
#pragma unroll
          for (int c = 1; c < PANEL_NB; ++c)
            if (c == j) a = v[r][c];
          a = a < T(0) ? -a : a;
          if (a > best || (a == best && rows[r] < bidx)) {
            best = a;
            bidx = rows[r];
          }
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        T ob = __shfl_down_sync(0xffffffffu, best, off);
        int64_t oi = __shfl_down_sync(0xffffffffu, bidx, off);
        if (ob > best || (ob == best && oi < bidx)) {
          best = ob;
          bidx = oi;
        }
      }
    } else {
      using PO = PivotOps<double>;
      PO::V key = PO::none();
      long long kidx = LLONG_MAX;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        if (rows[r] < m && rows[r] >= j) {
          T a = v[r][0];
#pragma unroll
          for (int c = 1; c < PANEL_NB; ++c)
            if (c == j) a = v[r][c];
          const PO::V k = PO::mag(a);
          if (PO::better(k, key, rows[r], kidx)) {
            key = k;
            kidx = rows[r];
          }
        }
      }
      PO::argmax(key, kidx);
      best = PO::carry(key);
      bidx = kidx == LLONG_MAX ? INT64_MAX : kidx;
    }
    if (lane == 0) {
      s_val[warp] = best;
      s_idx[warp] = bidx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      T bb = s_val[0];
      int64_t bi = s_idx[0];
      for (int w = 1; w < PANEL_THREADS / 32; ++w)
        if (panel_better<T>(s_val[w], bb, s_idx[w], bi)) {
          bb = s_val[w];
          bi = s_idx[w];
        }
      s_best = bi;
      T *slot = cand + ((int64_t)par * nblocks + blockIdx.x) * W;
      slot[PANEL_NB] = bb;
      slot[PANEL_NB + 1] = (T)(double)(bi == INT64_MAX ? -1 : bi);
    }
    __syncthreads();
    // the owner thread of the block's best row publishes the row
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (rows[r] == s_best) {
        T *slot = cand + ((int64_t)par * nblocks + blockIdx.x) * W;
#pragma unroll
        for (int c = 0; c < PANEL_NB; ++c) slot[c] = v[r][c];
      }
      if (rows[r] == j) {
        T *rb = rowj_buf + (int64_t)par * PANEL_NB;
#pragma unroll
        for (int c = 0; c < PANEL_NB; ++c) rb[c] = v[r][c];
      }
    }
    // ---- 2. grid barrier
    if (!grid_barrier(bar, nblocks, status, 100 + j)) return;
    // ---- 3. global pivot (same in every block)
    if (threadIdx.x < 32) {
      T bb = panel_none<T>();
      int64_t bi = INT64_MAX;
      for (unsigned b = lane; b < nblocks; b += 32) {
        const T *slot = cand + ((int64_t)par * nblocks + b) * W;
        T val = __ldcg(slot + PANEL_NB);
        int64_t idx = (int64_t)__ldcg(slot + PANEL_NB + 1);
        if (idx >= 0 && panel_better<T>(val, bb, idx, bi)) {
          bb = val;
          bi = idx;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        T ob = __shfl_down_sync(0xffffffffu, bb, off);
        int64_t oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (panel_better<T>(ob, bb, oi, bi)) {
          bb = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        // IAMAX starts from |a_jj| and only a larger value moves it: a NaN at
        // row j (or no comparable entry at all) keeps row j (-1 below)
        const T ajj = __ldcg(rowj_buf + (int64_t)par * PANEL_NB + j);
        s_p = (bi == INT64_MAX || ajj != ajj) ? -1 : bi;
      }
    }
    __syncthreads();
    const bool none = s_p < 0;
    const int64_t p = none ? (int64_t)j : s_p;  // keep row j, as a first-index IAMAX does
    const unsigned owner = (unsigned)((p % nthreads) / PANEL_THREADS);
    if (threadIdx.x < PANEL_NB) {
      const T oj = __ldcg(rowj_buf + (int64_t)par * PANEL_NB + threadIdx.x);
      s_u[threadIdx.x] =
          none ? oj : __ldcg(cand + ((int64_t)par * nblocks + owner) * W + threadIdx.x);
      s_oldj[threadIdx.x] = oj;
    }
    __syncthreads();
    T piv = s_u[0];
#pragma unroll
    for (int c = 1; c < PANEL_NB; ++c)
      if (c == j) piv = s_u[c];
    const T apiv = piv < T(0) ? -piv : piv;
    const bool nonzero = piv != T(0);
    // getf2_k.c:103-116: scale (and swap the processed columns) only when
    // |pivot| >= DBL_MIN.  Columns after j always see the interchange, as the
    // reference applies the recorded pivots lazily to later columns.
    const bool scaled = nonzero && apiv >= tiny_pivot<T>();
    const bool swap = p != j;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      ipiv[j] = (int)(p + row_off + 1);
      if (!nonzero && *info == 0) *info = (int)(j + row_off + 1);
    }
    // FP64: one division per warp, broadcast (a division is ~10 FP64 operations)
    T rcp = T(1);
    if (sizeof(T) == 8) {
      if (lane == 0 && scaled) rcp = T(1) / piv;
      rcp = __shfl_sync(0xffffffffu, rcp, 0);
    } else if (scaled) {
      rcp = T(1) / piv;
    }
    // ---- 4. interchange and update the rows this thread owns
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int64_t i = rows[r];
      if (i >= m || i < j) continue;
      if (swap && i == j) {
#pragma unroll
        for (int c = 0; c < PANEL_NB; ++c)
          if (scaled || c > j) v[r][c] = s_u[c];
        continue;  // the pivot row is final
      }
      if (swap && i == p) {
#pragma unroll
        for (int c = 0; c < PANEL_NB; ++c)
          if (scaled || c > j) v[r][c] = s_oldj[c];
      }
      if (i == j) continue;
      T l = v[r][0];
#pragma unroll
      for (int c = 1; c < PANEL_NB; ++c)
        if (c == j) l = v[r][c];
      if (scaled) l *= rcp;
#pragma unroll
      for (int c = 0; c < PANEL_NB; ++c) {
        if (c == j) v[r][c] = l;
        if (c > j) v[r][c] = fma(-l, s_u[c], v[r][c]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (rows[r] < m)
#pragma unroll
      for (int c = 0; c < PANEL_NB; ++c)
        if (c < nb) A[rows[r] + c * lda] = v[r][c];
}


// Row interchanges (lapack/laswp/generic/laswp_k_1.c semantics): rows
// k1..k2 (1-based) in order for incx > 0, in reverse for incx < 0; the pivot
// of row i is ipiv[(k1-1) + (i-k1)*|incx|].  One thread per column applies the
// interchanges in sequence (each column is independent).
template <typename T>
__global__ void laswp_kernel(int64_t n, T *__restrict__ A, int64_t lda, int64_t k1, int64_t k2,
                             const int *__restrict__ ipiv, int64_t incx) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= n) return;
  T *a = A + col * lda;
  const int64_t cnt = k2 - k1 + 1;
  const int64_t ainc = incx < 0 ? -incx : incx;
  for (int64_t t = 0; t < cnt; ++t) {
    const int64_t i = incx > 0 ? k1 + t : k2 - t;
    const int64_t ip = ipiv[(k1 - 1) + (i - k1) * ainc];
    if (ip != i) {
      T tmp = a[i - 1];
      a[i - 1] = a[ip - 1];
      a[ip - 1] = tmp;
    }
  }
}

// Final permutation of a pivot sequence: row i of P*B is row perm[i] of B.
// One thread replays the interchanges on an index vector (only used for
// the solve step, where it replaces many sequential column sweeps).
__global__ void pivots_to_perm_kernel(int64_t n, const int *__restrict__ ipiv,
                                      int *__restrict__ perm) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int64_t i = 0; i < n; ++i) perm[i] = (int)i;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t ip = ipiv[i] - 1;
    if (ip != i) {
      int t = perm[i];
      perm[i] = perm[ip];
      perm[ip] = t;
    }
  }
}

template <typename T>
__global__ void permute_rows_kernel(int64_t n, int64_t ncol, const int *__restrict__ perm,
                                    const T *__restrict__ src, int64_t lds, T *__restrict__ dst,
                                    int64_t ldd, int inverse) {
  const int64_t total = n * ncol;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e / n, i = e - c * n;
    if (!inverse)
      dst[i + c * ldd] = src[perm[i] + c * lds];
    else
      dst[perm[i] + c * ldd] = src[i + c * lds];
  }
}

// Unblocked Cholesky of an nb x nb diagonal block (nb <= PANEL_NB) in
// shared memory: lapack/potf2/potf2_L.c:50-97's algorithm (upper: potf2_U.c,
// handled by transposing into the lower form), right-looking: column j's
// pivot is a_jj less the updates already applied, its square root and one
// reciprocal come from one thread, the column is scaled by it and every
// thread takes a share of the rank-1 update of the trailing triangle.  (The
// dot-product form ran one serial chain of up to nb FP64 FMAs per row in a
// single warp, and a division in every thread, on the FP64 pipe that this
// part has least of: 70 us per 32 x 32 block.)  On the first pivot <= 0 the
// pivot value is written back and info = row_off + j + 1; later calls see
// info != 0 and return at once.
template <typename T>
__global__ void __launch_bounds__(256)
potf2_kernel(int upper, int nb, T *__restrict__ A, int64_t lda, int *__restrict__ info,
             int64_t row_off) {
  if (*info) return;
  __shared__ T S[PANEL_NB][PANEL_NB + 1];  // lower-triangular working copy
  __shared__ int s_fail;
  __shared__ T s_rcp;
  const int tid = threadIdx.x;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    int r = e % nb, c = e / nb;
    if (r >= c) S[r][c] = upper ? A[c + (int64_t)r * lda] : A[r + (int64_t)c * lda];
  }
  if (tid == 0) s_fail = -1;
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (tid == 0) {
      const T ajj = S[j][j];
      if (ajj <= T(0)) {
        s_fail = j;
      } else {
        const T d = sqrt(ajj);
        S[j][j] = d;
        s_rcp = T(1) / d;
      }
    }
    __syncthreads();
    if (s_fail >= 0) break;
    const T r = s_rcp;
    for (int i = j + 1 + tid; i < nb; i += blockDim.x) S[i][j] *= r;
    __syncthreads();
    // S[i][k] -= l_ij l_kj for j < k <= i < nb
    const int m = nb - j - 1;
    for (int e = tid; e < m * m; e += blockDim.x) {
      const int ii = e % m, kk = e / m;
      if (kk > ii) continue;
      const int i = j + 1 + ii, k = j + 1 + kk;
      S[i][k] = fma(-S[i][j], S[k][j], S[i][k]);
    }
    __syncthreads();
  }
  const int ncols = s_fail >= 0 ? s_fail + 1 : nb;
  for (int e = tid; e < nb * nb; e += blockDim.x) {
    int r = e % nb, c = e / nb;
    if (r < c || c >= ncols) continue;
    if (s_fail >= 0 && c == s_fail && r != c) continue;  // column stops at the failing pivot
    if (upper)
      A[c + (int64_t)r * lda] = S[r][c];
    else
      A[r + (int64_t)c * lda] = S[r][c];
  }
  if (tid == 0 && s_fail >= 0) *info = (int)(row_off + s_fail + 1);
}

constexpr int CPANEL_THREADS = 512;
constexpr int CPANEL_WARPS = CPANEL_THREADS / 32;
constexpr int CPANEL_MAX_CS = 16;       // one pushing warp per destination CTA

// Shared memory of the cluster panel kernel: candidate inboxes (rows,
// values, indices), per-warp candidate rows and row j, by column parity, and
// the two inbox mbarriers.
template <typename T>
__host__ __device__ constexpr size_t cpanel_smem_bytes() {
  return (size_t)2 * (2 * CPANEL_MAX_CS + 2) * PANEL_NB * sizeof(T)  // inbox + warp rows, row j x2
         + (size_t)2 * (CPANEL_MAX_CS + CPANEL_WARPS) * sizeof(T)     // inbox/warp values
         + (size_t)2 * CPANEL_MAX_CS * sizeof(int) + 8                // inbox row indices
         + (size_t)2 * CPANEL_WARPS * sizeof(long long) + 64          // warp row indices
         + 2 * sizeof(unsigned long long) + 8;                        // inbox mbarriers
}

// First maximum of (value, row) pairs over a warp: the largest value, the
// lowest row among equal values (IAMAX order).  An empty entry is (-1,
// LLONG_MAX).  Every lane receives the result.
template <typename T>
__device__ __forceinline__ void warp_argmax(T &v, long long &i) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const T ov = __shfl_xor_sync(0xffffffffu, v, off);
    const long long oi = __shfl_xor_sync(0xffffffffu, i, off);
    if (ov > v || (ov == v && oi < i)) {
      v = ov;
      i = oi;
    }
  }
}
// FP32: the bits of a non-negative float order like the value, so the
// maximum is one integer reduction and the first row among the maxima a
// second (rows < 2^31).
template <>
__device__ __forceinline__ void warp_argmax<float>(float &v, long long &i) {
  const unsigned key = v < 0.f ? 0u : __float_as_uint(v) + 1u;
  const unsigned kmax = __reduce_max_sync(0xffffffffu, key);
  const unsigned ik = key == kmax ? (unsigned)i : 0xffffffffu;
  const unsigned imin = __reduce_min_sync(0xffffffffu, ik);
  v = kmax == 0u ? -1.f : __uint_as_float(kmax - 1u);
  i = imin == 0xffffffffu ? LLONG_MAX : (long long)imin;
}
__device__ __forceinline__ void PivotOps<float>::argmax(V &v, long long &i) {
  warp_argmax<float>(v, i);
}

// Distributed-shared-memory messages of the cluster panel.  A value is stored
// into another CTA's shared memory with st.async, which completes its bytes on
// that CTA's mbarrier; the receiver waits on its own mbarrier only.
__device__ __forceinline__ uint32_t cl_smem_addr(const void *local, int rank) {
  uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(local)), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_async(uint32_t dst, float v, uint32_t mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];"
               ::"r"(dst), "r"(__float_as_uint(v)), "r"(mbar) : "memory");
}
__device__ __forceinline__ void st_async(uint32_t dst, double v, uint32_t mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];"
               ::"r"(dst), "l"((unsigned long long)__double_as_longlong(v)), "r"(mbar)
               : "memory");
}
__device__ __forceinline__ void st_async(uint32_t dst, int v, uint32_t mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];"
               ::"r"(dst), "r"(v), "r"(mbar) : "memory");
}


__device__ __forceinline__ void cl_mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;"
               ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(bar))), "r"(count)
               : "memory");
}
__device__ __forceinline__ void cl_mbar_expect(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(bar))), "r"(bytes)
               : "memory");
}
// Wait (acquire, cluster scope) for the phase of `parity` of a local
// mbarrier; false after about `limit_ns` nanoseconds.
__device__ __forceinline__ bool cl_mbar_wait(unsigned long long *bar, unsigned parity,
                                             unsigned long long limit_ns) {
  const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
  unsigned long long t0 = 0;
  for (unsigned i = 0;; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok) : "r"(a), "r"(parity) : "memory");
    if (ok) return true;
    if ((i & 63u) == 0) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (i == 0) t0 = t;
      else if (t - t0 > limit_ns) return false;
    }
  }
}
constexpr unsigned long long CPANEL_WAIT_NS = 2000000000ull;  // 2 s: never expected

// Panel LU on one thread-block cluster (up to 16 CTAs of 512 threads).
// Same algorithm and pivot rules as getf2_panel_kernel.  Each thread keeps
// its L panel rows in registers (updates are predicated FMAs with
// compile-time column indices; the pivot row is read with 16-byte shared
// loads).  Per column: after one CTA barrier every warp knows the CTA's
// candidate (first maximum of column j over its rows), and warp w sends that
// candidate -- value, row index and the 32-element row -- into CTA w's inbox
// with st.async (row j is sent the same way by the CTA that holds it).  Each
// store completes its bytes on the receiving CTA's inbox mbarrier, so a CTA
// waits for exactly its own CS messages and never for the whole cluster.
// Inboxes and mbarriers alternate between two buffers by column parity.  A
// buffer is written again two columns later; a CTA can only send for column
// j+2 after it received every column j+1 message, and each CTA sends its
// column j+1 messages after all its warps passed the CTA barrier of column
// j+1, i.e. after they finished reading the column-j buffer.  Every wait is
// bounded: a CTA that gives up records GB_KERR_CLUSTER_TIMEOUT, stops, waits
// (bounded) for the messages of the columns it armed, and meets the others
// at the final cluster barrier.
template <typename T, int L, int NB>
__global__ void __launch_bounds__(CPANEL_THREADS, 1)
getf2_cluster_kernel(int64_t m, int nb, T *__restrict__ A, int64_t lda, int *__restrict__ ipiv,
                     int64_t row_off, int *__restrict__ info, int *__restrict__ status) {
  static_assert(NB <= PANEL_NB && NB % 4 == 0, "one lane per panel column");
  static_assert(CPANEL_WARPS == CPANEL_MAX_CS, "one sending warp per destination CTA");
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *in_row = reinterpret_cast<T *>(smem_raw);                 // [2][CS][NB] candidates
  T *w_row = in_row + 2 * CPANEL_MAX_CS * PANEL_NB;             // [2][WARPS][NB] warp bests
  T *in_rowj = w_row + 2 * CPANEL_WARPS * PANEL_NB;             // [2][NB] row j (inbox)
  T *j_slot = in_rowj + 2 * PANEL_NB;                           // [2][NB] row j (staged)
  T *in_val = j_slot + 2 * PANEL_NB;                            // [2][CS]
  T *red_val = in_val + 2 * CPANEL_MAX_CS;                      // [2][WARPS]
  int *in_idx = reinterpret_cast<int *>(red_val + 2 * CPANEL_WARPS);  // [2][CS]
  long long *red_idx = reinterpret_cast<long long *>(
      (reinterpret_cast<uintptr_t>(in_idx + 2 * CPANEL_MAX_CS) + 7) & ~uintptr_t(7));  // [2][WARPS]
  unsigned long long *mbar = reinterpret_cast<unsigned long long *>(
      red_idx + 2 * CPANEL_WARPS);                                                    // [2]
  __shared__ int s_abort;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // rows are dealt to the cluster's threads round robin: row r sits with
  // thread (r mod nthr), register slot (r div nthr).  nthr is a power of two
  // (the cluster size is), so both are a mask and a shift
  const int64_t nthr = (int64_t)CS * CPANEL_THREADS;
  const int lg_nthr = __ffsll(nthr) - 1;
  const int64_t nmask = nthr - 1;
  const int64_t g = (int64_t)rank * CPANEL_THREADS + tid;
  const int ncol = (int)(nb < m ? nb : m);
  // bytes one CTA receives per column: CS candidates (row, value, index) and row j
  const unsigned expect_bytes =
      (unsigned)(CS * (NB * sizeof(T) + sizeof(T) + sizeof(int)) + NB * sizeof(T));

  T r[L][NB];
#pragma unroll
  for (int q = 0; q < L; ++q) {
    const int64_t row = g + q * nthr;
#pragma unroll
    for (int c = 0; c < NB; ++c) r[q][c] = (row < m && c < nb) ? A[row + c * lda] : T(0);
  }
  if (tid == 0) {
    s_abort = 0;
    cl_mbar_init(&mbar[0], 1);
    cl_mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    // arm the buffers of columns 0 and 1
    if (ncol > 0) cl_mbar_expect(&mbar[0], expect_bytes);
    if (ncol > 1) cl_mbar_expect(&mbar[1], expect_bytes);
  }
  cluster.sync();  // every CTA's mbarriers are armed before anyone sends

  // 32 values of one register row into shared memory, 16 bytes at a time
  auto stage_row = [&](T *dst, const T (&src)[NB]) {
    if (sizeof(T) == 4) {
#pragma unroll
      for (int c = 0; c < NB; c += 4)
        *reinterpret_cast<float4 *>(dst + c) =
            make_float4((float)src[c], (float)src[c + 1], (float)src[c + 2], (float)src[c + 3]);
    } else {
#pragma unroll
      for (int c = 0; c < NB; c += 2)
        *reinterpret_cast<double2 *>(dst + c) = make_double2((double)src[c], (double)src[c + 1]);
    }
  };

  int armed_to = ncol < 2 ? ncol : 2;  // columns whose inbox phase has been armed
  int waited = 0;                      // columns whose messages have all arrived here
  bool ok = true;
  // fully unrolled over the NB columns: every register index and the
  // length of each row update (NB - 1 - j FMAs) are compile-time constants
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    if (j >= ncol) break;
    const int par = j & 1;
    // ---- local first maximum of |a_ij| over this thread's rows >= j
    using PO = PivotOps<T>;
    using V = typename PO::V;
    V best = PO::none();
    long long bidx = LLONG_MAX;
    if constexpr (sizeof(T) == 4) {
#pragma unroll
      for (int q = 0; q < L; ++q) {
        const int64_t row = g + q * nthr;
        if (row < m && row >= j) {
          T a = r[q][j];  // j is a compile-time index in the unrolled loop
          a = a < T(0) ? -a : a;
          if (a > best || (a == best && row < bidx)) {
            best = a;
            bidx = row;
          }
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < L; ++q) {
        const int64_t row = g + q * nthr;
        if (row < m && row >= j) {
          const V a = PO::mag(r[q][j]);
          if (PO::better(a, best, row, bidx)) {
            best = a;
            bidx = row;
          }
        }
      }
    }
    PO::argmax(best, bidx);
    // the lane holding the warp's best row stages it; the holder of row j too
    if (bidx != LLONG_MAX && (int)(bidx & 31) == lane) {
      const int qb = (int)(bidx >> lg_nthr);
#pragma unroll
      for (int q = 0; q < L; ++q)
        if (q == qb) stage_row(w_row + (par * CPANEL_WARPS + warp) * PANEL_NB, r[q]);
    }
    if (lane == 0) {
      red_val[par * CPANEL_WARPS + warp] = PO::carry(best);
      red_idx[par * CPANEL_WARPS + warp] = bidx;
    }
    const int jowner = (int)(((int64_t)j & nmask) / CPANEL_THREADS);
    if (jowner == rank && (int)(((int64_t)j & nmask) - (int64_t)rank * CPANEL_THREADS) == tid) {
      const int qj = (int)((int64_t)j >> lg_nthr);
#pragma unroll
      for (int q = 0; q < L; ++q)
        if (q == qj) stage_row(j_slot + par * PANEL_NB, r[q]);
    }
    __syncthreads();
    if (s_abort) {
      ok = false;
      break;
    }
    // ---- every warp: the CTA's candidate; warp w sends it (and row j) to CTA w
    V cb = lane < CPANEL_WARPS ? PO::uncarry(red_val[par * CPANEL_WARPS + lane]) : PO::none();
    long long ci = lane < CPANEL_WARPS ? red_idx[par * CPANEL_WARPS + lane] : LLONG_MAX;
    PO::argmax(cb, ci);
    if (warp < CS) {
      const int dst = warp;
      T rv = T(0);
      if (ci != LLONG_MAX && lane < NB) {
        const int wb = (int)(((ci & nmask) - (int64_t)rank * CPANEL_THREADS) >> 5);
        rv = w_row[(par * CPANEL_WARPS + wb) * PANEL_NB + lane];
      }
      const uint32_t rb = cl_smem_addr(&mbar[par], dst);
      if (lane < NB)
        st_async(cl_smem_addr(in_row + (par * CPANEL_MAX_CS + rank) * PANEL_NB + lane, dst), rv,
                 rb);
      if (lane == 0) {
        st_async(cl_smem_addr(in_val + par * CPANEL_MAX_CS + rank, dst), PO::carry(cb), rb);
        st_async(cl_smem_addr(in_idx + par * CPANEL_MAX_CS + rank, dst),
                 ci == LLONG_MAX ? -1 : (int)ci, rb);
      }
      if (jowner == rank && lane < NB)
        st_async(cl_smem_addr(in_rowj + par * PANEL_NB + lane, dst), j_slot[par * PANEL_NB + lane],
                 rb);
    }
    // ---- this CTA's inbox for column j is complete.  A thread that gives up
    // raises s_abort and carries on with whatever the inbox holds (every index
    // below stays in range); the whole CTA stops together after the next CTA
    // barrier, before any message of the next column is sent.
    const bool arrived = cl_mbar_wait(&mbar[par], (unsigned)((j >> 1) & 1), CPANEL_WAIT_NS);
    if (!arrived) {
      if (status) {
        atomicCAS(status, 0, GB_KERR_CLUSTER_TIMEOUT);
        atomicExch(status + 1, 200 + j);
      }
      s_abort = 1;
    } else {
      waited = j + 1;
    }
    if (arrived && tid == 0 && j + 2 < ncol) {
      cl_mbar_expect(&mbar[par], expect_bytes);  // re-arm this buffer for column j + 2
      armed_to = j + 3;
    }
    // ---- global pivot from the local inbox (identical in every CTA)
    V gb = PO::none();
    long long gi = LLONG_MAX;
    if (lane < CS) {
      const int idx = in_idx[par * CPANEL_MAX_CS + lane];
      if (idx >= 0) {
        gb = PO::uncarry(in_val[par * CPANEL_MAX_CS + lane]);
        gi = idx;
      }
    }
    PO::argmax(gb, gi);
    const T *rowj_v = in_rowj + par * PANEL_NB;
    // IAMAX starts from |a_jj| and only a larger value moves it: a NaN at row
    // j (or no comparable entry at all) keeps row j
    const T ajj = rowj_v[j];
    const bool keep = gi == LLONG_MAX || (sizeof(T) == 4 ? ajj != ajj : PO::is_nan(ajj));
    const int64_t p = keep ? (int64_t)j : gi;
    const T *u_v = keep ? rowj_v
                        : in_row + (par * CPANEL_MAX_CS + (int)((gi & nmask) / CPANEL_THREADS)) *
                                       PANEL_NB;
    const T piv = u_v[j];
    // piv != 0 (NaN counts) and |piv| >= the smallest normal (NaN does not);
    // FP32 keeps the float tests (the same results: the compiler then keeps
    // more of the 16-column kernel's rows in registers)
    const T apiv = piv < T(0) ? -piv : piv;
    const bool nonzero = sizeof(T) == 4 ? piv != T(0) : PO::nonzero(piv);
    const bool scaled =
        sizeof(T) == 4 ? (nonzero && apiv >= tiny_pivot<T>()) : PO::scaled(piv);  // getf2_k.c:103-116
    const bool swap = p != j;
    if (rank == 0 && tid == 0) {
      ipiv[j] = (int)(p + row_off + 1);
      if (!nonzero && *info == 0) *info = (int)(j + row_off + 1);
    }
    // FP64: one division per warp, broadcast (a division is ~10 FP64 operations)
    T rcp = T(1);
    if (sizeof(T) == 8) {
      if (lane == 0 && scaled) rcp = T(1) / piv;
      rcp = __shfl_sync(0xffffffffu, rcp, 0);
    } else if (scaled) {
      rcp = T(1) / piv;
    }
#pragma unroll
    for (int q = 0; q < L; ++q) {
      const int64_t i = g + q * nthr;
      if (i >= m || i < j) continue;
      if (swap && i == j) {
#pragma unroll
        for (int c = 0; c < NB; ++c)
          if (scaled || c > j) r[q][c] = u_v[c];
        continue;  // the pivot row is final
      }
      const bool take_j = swap && i == p;  // row p receives the old row j
      if (take_j) {
#pragma unroll
        for (int c = 0; c < NB; ++c)
          if (scaled || c > j) r[q][c] = rowj_v[c];
      }
      if (i == j) continue;
      T l = take_j ? rowj_v[j] : r[q][j];
      if (scaled) l *= rcp;
#pragma unroll
      for (int c = 0; c < NB; c += 4) {
        T u4[4];
        if (sizeof(T) == 4) {
          const float4 f = *reinterpret_cast<const float4 *>(u_v + c);
          u4[0] = (T)f.x; u4[1] = (T)f.y; u4[2] = (T)f.z; u4[3] = (T)f.w;
        } else {
          const double2 d0 = *reinterpret_cast<const double2 *>(u_v + c);
          const double2 d1 = *reinterpret_cast<const double2 *>(u_v + c + 2);
          u4[0] = (T)d0.x; u4[1] = (T)d0.y; u4[2] = (T)d1.x; u4[3] = (T)d1.y;
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int cc = c + t;
          if (cc == j) r[q][cc] = l;
          else if (cc > j) r[q][cc] = fma(-l, u4[t], r[q][cc]);
        }
      }
    }
  }
  __syncthreads();
  ok = ok && !s_abort;  // uniform across the CTA after the barrier
  if (ok) {
#pragma unroll
    for (int q = 0; q < L; ++q) {
      const int64_t row = g + q * nthr;
      if (row >= m) continue;
#pragma unroll
      for (int c = 0; c < NB; ++c)
        if (c < nb) A[row + c * lda] = r[q][c];
    }
  } else {
    // gave up: let the messages of every armed column land (bounded) before
    // this CTA's shared memory can go away
    if (tid == 0)
      for (int jj = waited; jj < armed_to; ++jj)
        cl_mbar_wait(&mbar[jj & 1], (unsigned)((jj >> 1) & 1), CPANEL_WAIT_NS / 8);
  }
  cluster.sync();  // no CTA leaves while another may still write into its inbox
}

template <typename T>
struct ClusterPanel {
  int max_cs = 0;  // largest launchable cluster size (0: unavailable)
  int lmax = 0;    // register rows per thread of the 32-column kernel
  int lmax16 = 0;  // register rows per thread of the 16-column kernel (FP32 only; 0: none)
};

// Rows per thread held in registers: 32 columns x 2 rows (FP32) or 1 row
// (FP64); for taller FP32 panels, 16 columns x 4 rows (FP64 panels taller
// than one cluster holds take the grid-wide kernel: a 16-column FP64 form
// measured slower, LU 16384 430 -> 455 ms).
template <typename T>
constexpr int cpanel_lmax() { return sizeof(T) == 4 ? 2 : 1; }
template <typename T>
constexpr int cpanel_lmax16() { return sizeof(T) == 4 ? 4 : 0; }

template <typename T>
void cpanel_allow_large_clusters() {
  cudaFuncSetAttribute(getf2_cluster_kernel<T, 1, PANEL_NB>,
                       cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if constexpr (cpanel_lmax<T>() > 1)
    cudaFuncSetAttribute(getf2_cluster_kernel<T, cpanel_lmax<T>(), PANEL_NB>,
                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if constexpr (cpanel_lmax16<T>() > 0)
    cudaFuncSetAttribute(getf2_cluster_kernel<T, cpanel_lmax16<T>(), 16>,
                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaGetLastError();
}

// Largest cluster size with at least one co-resident cluster of `kern`.
template <typename K>
int largest_cluster(K kern, size_t smem) {
  for (int cs = 16; cs >= 2; cs /= 2) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(CPANEL_THREADS);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters >= 1)
      return cs;
    cudaGetLastError();
  }
  return 0;
}

// Largest cluster the panel kernel launches with on the current device.
template <typename T>
ClusterPanel<T> probe_cluster_panel() {
  ClusterPanel<T> caps;
  const size_t smem = cpanel_smem_bytes<T>();
  cpanel_allow_large_clusters<T>();
  caps.max_cs = largest_cluster(getf2_cluster_kernel<T, cpanel_lmax<T>(), PANEL_NB>, smem);
  caps.lmax = caps.max_cs >= 2 ? cpanel_lmax<T>() : 0;
  if constexpr (cpanel_lmax16<T>() > 0) {
    // the 16-column kernel is used only with the same cluster size
    if (caps.max_cs >= 2 &&
        largest_cluster(getf2_cluster_kernel<T, cpanel_lmax16<T>(), 16>, smem) >= caps.max_cs)
      caps.lmax16 = cpanel_lmax16<T>();
  }
  if (config().verbose)
    fprintf(stderr,
            "libgbblas: cluster panel (%s): max cluster %d CTAs, %d rows/thread (32 columns), "
            "%d rows/thread (16 columns)\n",
            sizeof(T) == 4 ? "fp32" : "fp64", caps.max_cs, caps.lmax, caps.lmax16);
  return caps;
}

// The probe's result, found once per device.
template <typename T>
ClusterPanel<T> cluster_panel_caps() {
  static PerDeviceValue<ClusterPanel<T>> cache;
  return cache.get(current_device(), [] { return probe_cluster_panel<T>(); });
}

// Widest leaf (32 or 16 columns) whose cluster panel holds `rows` rows; 32
// when neither does (the grid-wide kernel then takes 32 columns).  (16-column
// leaves for every FP64 panel were tried: more leaves, each as slow -- the
// per-column exchange, not the FP64 rank-1 updates, sets a leaf's time --
// and the recursion's extra small updates: emulated-update LU 8192 147 ->
// 175 ms.)
template <typename T>
int lu_leaf_width(int64_t rows) {
  const ClusterPanel<T> caps = cluster_panel_caps<T>();
  if (caps.max_cs < 2) return PANEL_NB;
  const int64_t cap32 = (int64_t)caps.max_cs * CPANEL_THREADS * caps.lmax;
  const int64_t cap16 = (int64_t)caps.max_cs * CPANEL_THREADS * caps.lmax16;
  return (rows > cap32 && rows <= cap16) ? 16 : PANEL_NB;
}

// Launch the cluster panel when the panel fits one cluster; returns 1 when
// it does not (the caller then uses the grid-wide kernel).
template <typename T>
int launch_cluster_panel(int64_t rows, int nb, T *A, int64_t lda, int *ipiv, int64_t row_off,
                         int *info, int *status, cudaStream_t s) {
  const ClusterPanel<T> caps = cluster_panel_caps<T>();
  if (caps.max_cs < 2) return 1;
  int64_t cs = (rows + CPANEL_THREADS - 1) / CPANEL_THREADS;
  if (cs < 2) cs = 2;
  if (cs > caps.max_cs) cs = caps.max_cs;
  const int64_t L = (rows + cs * CPANEL_THREADS - 1) / (cs * CPANEL_THREADS);
  // 16-column panels may take up to lmax16 rows per thread
  const bool narrow = nb <= 16 && L > caps.lmax && L <= caps.lmax16;
  if (L > caps.lmax && !narrow) return 1;
  // cluster sizes must divide the grid; use a power of two
  int csp = 2;
  while (csp < cs) csp *= 2;
  if (csp > caps.max_cs) return 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)csp);
  cfg.blockDim = dim3(CPANEL_THREADS);
  cfg.dynamicSmemBytes = cpanel_smem_bytes<T>();
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csp;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  count_launch();
  cudaError_t e = cudaErrorInvalidValue;
  if (narrow) {
    if constexpr (cpanel_lmax16<T>() > 0)
      e = cudaLaunchKernelEx(&cfg, getf2_cluster_kernel<T, cpanel_lmax16<T>(), 16>, rows, nb, A,
                             lda, ipiv, row_off, info, status);
  } else if (L == 1) {
    e = cudaLaunchKernelEx(&cfg, getf2_cluster_kernel<T, 1, PANEL_NB>, rows, nb, A, lda, ipiv,
                           row_off, info, status);
  } else {
    if constexpr (cpanel_lmax<T>() > 1)
      e = cudaLaunchKernelEx(&cfg, getf2_cluster_kernel<T, cpanel_lmax<T>(), PANEL_NB>, rows, nb,
                             A, lda, ipiv, row_off, info, status);
  }
  return check_cuda(e, "cluster panel launch");
}

template <typename T, int R>
int launch_panel(int64_t rows, int nb, T *A, int64_t lda, int *ipiv, int64_t row_off, int *info,
                 T *slots, unsigned *bar, int *status, unsigned nblocks, cudaStream_t s) {
  void *args[] = {&rows, &nb, &A, &lda, &ipiv, &row_off, &info, &slots, &bar, &status};
  count_launch();
  return check_cuda(cudaLaunchCooperativeKernel((const void *)getf2_panel_kernel<T, R>,
                                                dim3(nblocks), dim3(PANEL_THREADS), args, 0, s),
                    "panel factorisation launch");
}

template <typename T, int R>
int coop_limit() {
  static PerDeviceValue<int> cache;
  return cache.get(current_device(), [] {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, getf2_panel_kernel<T, R>,
                                                      PANEL_THREADS, 0) != cudaSuccess) {
      cudaGetLastError();
      per_sm = 0;
    }
    const int lim = per_sm * sm_count();
    return lim > 0 ? lim : 1;
  });
}

template <typename T>
void gemm_minus(int64_t m, int64_t n, int64_t k, const T *A, int64_t lda, const T *B,
                int64_t ldb, T *C, int64_t ldc, cudaStream_t s);
template <>
void gemm_minus<double>(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda,
                        const double *B, int64_t ldb, double *C, int64_t ldc, cudaStream_t s) {
  launch_dgemm_fp64(0, 0, m, n, k, -1.0, A, lda, B, ldb, 1.0, C, ldc, s);
}

template <typename T>
int trsm_any(int side, int uplo, int trans, int unit, int64_t m, int64_t n, const T *A,
             int64_t lda, T *B, int64_t ldb, cudaStream_t s);
template <>
int trsm_any<double>(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                     const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s) {
  return dtrsm_device(side, uplo, trans, unit, m, n, 1.0, A, lda, B, ldb, s);
}
template <>
int trsm_any<float>(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                    const float *A, int64_t lda, float *B, int64_t ldb, cudaStream_t s) {
  return strsm_device(side, uplo, trans, unit, m, n, 1.0f, A, lda, B, ldb, s);
}

}  // namespace

// B := L^-1 B for the unit-lower L11 of an LU step (L n1 x n1, n1 <= 256;
// B n1 x w): the TRSM_ILTCOPY + TRSM_KERNEL_LT pair of the reference's
// getrf (driver/level3/trsm_L.c with the inverted diagonal of
// trsm_ltcopy), in one launch.  Each CTA owns 32 columns of B in shared
// memory; its warps first invert the 32 x 32 diagonal blocks of L11 (lane c
// solves for column c), then block row i of B gets B_i -= L_ik B_k (k < i,
// L tiles read from L2, coalesced) and B_i = inv(L_ii) B_i.  Rows past n1
// are identity padding.
constexpr int LT_COLS = 32;   // columns of B per CTA
constexpr int LT_MAXN = 256;  // largest L11

template <typename T>
__host__ __device__ constexpr size_t lu_trsm_smem(int nblk) {
  return (size_t)(2 * nblk + 1) * 32 * (LT_COLS + 1) * sizeof(T);  // B, inverses, one L tile
}

template <typename T>
__global__ void __launch_bounds__(256)
lu_trsm_kernel(int n1, int64_t w, const T *__restrict__ L, int64_t ldl, T *__restrict__ B,
               int64_t ldb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nblk = (n1 + 31) / 32;
  const int nr = nblk * 32;
  T *Bs = reinterpret_cast<T *>(smem_raw);  // [nr][LT_COLS + 1]
  T *Li = Bs + nr * (LT_COLS + 1);           // [nblk][32][33]: L_dd, then its inverse
  T *Lt = Li + nblk * 32 * 33;                // [32][33]: the current L_ik tile
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t c0 = (int64_t)blockIdx.x * LT_COLS;
  const int nc = (int)((w - c0) < LT_COLS ? (w - c0) : LT_COLS);
  for (int e = tid; e < nr * LT_COLS; e += 256) {
    const int r = e % nr, c = e / nr;
    Bs[r * (LT_COLS + 1) + c] = (r < n1 && c < nc) ? B[r + (c0 + c) * ldb] : T(0);
  }
  for (int d = warp; d < nblk; d += 8) {
    const int b0 = d * 32;
    T *Ld = Li + d * 32 * 33;
#pragma unroll 4
    for (int c = 0; c < 32; ++c) {
      const bool in = b0 + lane < n1 && b0 + c < n1;
      Ld[lane * 33 + c] = in ? L[(b0 + lane) + (int64_t)(b0 + c) * ldl] : T(lane == c ? 1 : 0);
    }
    __syncwarp();
    T x[32];  // column `lane` of inv(L_dd) (unit diagonal)
#pragma unroll
    for (int r = 0; r < 32; ++r) {
      T sum = (r == lane) ? T(1) : T(0);
#pragma unroll
      for (int k = 0; k < r; ++k) sum = fma(-Ld[r * 33 + k], x[k], sum);
      x[r] = sum;
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 32; ++r) Ld[r * 33 + lane] = x[r];
  }
  __syncthreads();
  const int r = lane, cg = warp;  // row r of a block, columns cg*4 .. cg*4+3
  for (int i = 0; i < nblk; ++i) {
    T acc[4] = {T(0), T(0), T(0), T(0)};
    for (int k = 0; k < i; ++k) {
      // stage L(i-block, k-block) once for all 32 columns of the CTA
      __syncthreads();
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = tid + 256 * u, rr = e & 31, cc = e >> 5;
        Lt[rr * 33 + cc] = (i * 32 + rr < n1) ? L[(int64_t)(i * 32 + rr) + (int64_t)(k * 32 + cc) * ldl]
                                              : T(0);
      }
      __syncthreads();
#pragma unroll 8
      for (int kk = 0; kk < 32; ++kk) {
        const T l = Lt[r * 33 + kk];
        const T *bk = Bs + (k * 32 + kk) * (LT_COLS + 1) + cg * 4;
#pragma unroll
        for (int t = 0; t < 4; ++t) acc[t] = fma(l, bk[t], acc[t]);
      }
    }
    T *bi = Bs + (i * 32 + r) * (LT_COLS + 1) + cg * 4;
#pragma unroll
    for (int t = 0; t < 4; ++t) bi[t] -= acc[t];
    __syncthreads();
    const T *Ld = Li + i * 32 * 33;
    T y[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      const T l = Ld[r * 33 + kk];
      const T *bk = Bs + (i * 32 + kk) * (LT_COLS + 1) + cg * 4;
#pragma unroll
      for (int t = 0; t < 4; ++t) y[t] = fma(l, bk[t], y[t]);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < 4; ++t) bi[t] = y[t];
    __syncthreads();
  }
  for (int e = tid; e < nr * LT_COLS; e += 256) {
    const int rr = e % nr, c = e / nr;
    if (rr < n1 && c < nc) B[rr + (c0 + c) * ldb] = Bs[rr * (LT_COLS + 1) + c];
  }
}

template <typename T>
int lu_trsm(int64_t n1, int64_t w, const T *L, int64_t ldl, T *B, int64_t ldb, cudaStream_t s) {
  if (n1 <= 0 || w <= 0) return GB_SUCCESS;
  if (n1 > LT_MAXN) return trsm_any<T>(0, 1, 0, 0, n1, w, L, ldl, B, ldb, s);
  const int nblk = (int)((n1 + 31) / 32);
  const size_t smem = lu_trsm_smem<T>(nblk);
  static PerDeviceOnce attr_once;
  const int ast = attr_once.run(current_device(), [] {
    GB_CUDA(cudaFuncSetAttribute(lu_trsm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)lu_trsm_smem<T>(LT_MAXN / 32)));
    return GB_SUCCESS;
  });
  if (ast) return ast;
  const int64_t grid = (w + LT_COLS - 1) / LT_COLS;
  { lu_trsm_kernel<T><<<(unsigned)grid, 256, smem, s>>>((int)n1, w, L, ldl, B, ldb); count_launch(); }
  return check_cuda(cudaGetLastError(), "lu_trsm");
}

// Interchange sequences of up to LASWP_FUSED_MAX steps in one launch, any
// incx.  Every CTA replays the sequence on slot indices in shared memory
// (slot s < cnt is row k1-1+s of the window; slot cnt+t stands for the pivot
// row of step t outside the window, deduplicated to its first step), which
// gives the final source of every touched row; the CTA then gathers the
// moved rows of its columns into shared memory and writes them back.  The
// result equals applying the interchanges one after another
// (lapack/laswp/generic/laswp_k_1.c), at the cost of two memory round trips
// instead of one per interchange.
constexpr int LASWP_FUSED_MAX = 512;
constexpr int LASWP_FUSED_ELEMS = 4096;

template <typename T>
__global__ void __launch_bounds__(256)
laswp_fused_kernel(int64_t n, T *__restrict__ A, int64_t lda, int64_t k1, int64_t k2,
                   const int *__restrict__ ipiv, int64_t incx, int cols_per_cta, int64_t skip0,
                   int64_t skipw) {
  __shared__ int prow[LASWP_FUSED_MAX];
  __shared__ int slotp[LASWP_FUSED_MAX];
  __shared__ int pos[2 * LASWP_FUSED_MAX];
  __shared__ int moved[2 * LASWP_FUSED_MAX];
  __shared__ int nmoved;
  __shared__ T vals[LASWP_FUSED_ELEMS];
  const int cnt = (int)(k2 - k1 + 1);
  const int64_t w0 = k1 - 1;
  const int64_t ainc = incx < 0 ? -incx : incx;
  const int tid = threadIdx.x;
  for (int t = tid; t < cnt; t += blockDim.x) {
    const int64_t i = incx > 0 ? k1 + t : k2 - t;  // 1-based row of step t
    prow[t] = ipiv[(k1 - 1) + (i - k1) * ainc] - 1;
  }
  for (int sl = tid; sl < 2 * cnt; sl += blockDim.x) pos[sl] = sl;
  if (tid == 0) nmoved = 0;
  __syncthreads();
  for (int t = tid; t < cnt; t += blockDim.x) {
    const int p = prow[t];
    int sp;
    if (p >= w0 && p < w0 + cnt) {
      sp = (int)(p - w0);
    } else {
      int c = t;
      for (int u = 0; u < t; ++u)
        if (prow[u] == p) {
          c = u;
          break;
        }
      sp = cnt + c;
    }
    slotp[t] = sp;
  }
  __syncthreads();
  if (tid == 0) {
    // pos[s] = slot whose original row ends up in slot s
    for (int t = 0; t < cnt; ++t) {
      const int si = incx > 0 ? t : cnt - 1 - t;
      const int sp = slotp[t];
      if (sp != si) {
        const int a = pos[si];
        pos[si] = pos[sp];
        pos[sp] = a;
      }
    }
  }
  __syncthreads();
  for (int sl = tid; sl < 2 * cnt; sl += blockDim.x) {
    const bool active = sl < cnt || slotp[sl - cnt] == sl;
    if (active && pos[sl] != sl) moved[atomicAdd(&nmoved, 1)] = sl;
  }
  __syncthreads();
  const int nm = nmoved;
  if (nm == 0) return;
  auto row_of = [&](int sl) -> int64_t { return sl < cnt ? w0 + sl : (int64_t)prow[sl - cnt]; };
  // the n columns visited are the matrix's columns with [skip0, skip0 + skipw) left out
  auto col_of = [&](int64_t c) -> int64_t { return c < skip0 ? c : c + skipw; };
  // the plan is reused for every column chunk this CTA visits; within a
  // chunk each thread keeps 8 loads in flight before it stores to shared
  const int64_t nchunks = (n + cols_per_cta - 1) / cols_per_cta;
  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int64_t c0 = ch * cols_per_cta;
    const int nc = (int)((n - c0) < cols_per_cta ? (n - c0) : cols_per_cta);
    const int total = nm * nc;
    for (int e0 = tid; e0 < total; e0 += 8 * 256) {
      T v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + u * 256;
        if (e < total) {
          const int c = e / nm, q = e - c * nm;
          v[u] = A[row_of(pos[moved[q]]) + col_of(c0 + c) * lda];
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (e0 + u * 256 < total) vals[e0 + u * 256] = v[u];
    }
    __syncthreads();
    for (int e = tid; e < total; e += 256) {
      const int c = e / nm, q = e - c * nm;
      A[row_of(moved[q]) + col_of(c0 + c) * lda] = vals[e];
    }
    __syncthreads();
  }
}

template <typename T>
int launch_laswp_fused(int64_t n, T *A, int64_t lda, int64_t k1, int64_t k2, const int *ipiv,
                       int64_t incx, cudaStream_t s, int64_t skip0 = INT64_MAX,
                       int64_t skipw = 0) {
  const int64_t cnt = k2 - k1 + 1;
  int cols = (int)(LASWP_FUSED_ELEMS / (2 * cnt));
  if (cols < 1) cols = 1;
  int64_t grid = (n + cols - 1) / cols;
  const int64_t cap = (int64_t)sm_count() * 2;
  if (grid > cap) grid = cap;
  { laswp_fused_kernel<T><<<(unsigned)grid, 256, 0, s>>>(n, A, lda, k1, k2, ipiv, incx, cols,
                                                         skip0, skipw); count_launch(); }
  return check_cuda(cudaGetLastError(), "laswp launch");
}

template <typename T>
int laswp_device(int64_t n, T *A, int64_t lda, int64_t k1, int64_t k2, const int *ipiv,
                 int64_t incx, cudaStream_t s) {
  if (n <= 0 || incx == 0 || k2 < k1) return GB_SUCCESS;
  if (k2 - k1 + 1 <= LASWP_FUSED_MAX) return launch_laswp_fused<T>(n, A, lda, k1, k2, ipiv, incx, s);
  { laswp_kernel<T><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(n, A, lda, k1, k2, ipiv, incx); count_launch(); }
  return check_cuda(cudaGetLastError(), "laswp launch");
}

// Recursive LU (lapack/getrf/getrf_single.c:47-180 splits the columns in
// halves in the same way): factor the left half, solve for U12 with the
// unit-lower L11, update A22 with one GEMM of rank n1 and factor A22
// recursively.  Leaves of PANEL_NB columns go to the panel kernels, and each
// leaf's interchanges are applied to all other columns right after it (see
// lu_panel), which puts every row where the reference's per-level LASWP
// calls put it.  Compared with a flat right-looking sweep, every trailing element
// is rounded O(log n) instead of O(n / PANEL_NB) times and the GEMMs are
// large, which matters most for the FP32 factorisation of the mixed solver.
template <typename T>
struct LuCtx {
  T *A;
  int64_t lda;
  int *ipiv;
  int *info;
  T *slots;
  unsigned *bar;
  int *status;
  int lim1, lim2;
  int gemm_mode;  // double only: 0 native FP64 updates, 1 emulated-FP64 updates
  int64_t nrows, ncols;          // the whole matrix
  int64_t blk0 = 0, blk1 = 0;    // columns a panel's interchanges reach (see lu_panel)
  bool use_cluster = true;  // panel on one thread-block cluster when it fits
  cudaStream_t s;
};


// The engine of a trailing update A22 -= A21 A12 of shape m x n x k: 1 for
// the tensor-core form (emulated FP64 / bf16x3 FP32), 0 for the FMA units.
// The look-ahead LU splits one update into column pieces and runs every
// piece on the engine the whole update would use, so each element gets the
// same arithmetic either way.
template <typename T>
int lu_update_engine(const LuCtx<T> &c, int64_t m, int64_t n, int64_t k);
template <>
int lu_update_engine<double>(const LuCtx<double> &c, int64_t m, int64_t n, int64_t k) {
  return (c.gemm_mode == 1 && m >= 256 && n >= 256 && k >= 64) ? 1 : 0;
}
template <>
int lu_update_engine<float>(const LuCtx<float> &, int64_t m, int64_t n, int64_t k) {
  const int mode = gb_get_sgemm_mode();
  return (mode == GB_SGEMM_TENSOR || (mode == GB_SGEMM_AUTO && m >= 1024 && n >= 1024 && k >= 64))
             ? 1 : 0;
}

template <typename T>
int lu_update(LuCtx<T> &c, int64_t m, int64_t n, int64_t k, const T *A21, const T *A12, T *A22,
              int engine = -1);
template <>
int lu_update<double>(LuCtx<double> &c, int64_t m, int64_t n, int64_t k, const double *A21,
                      const double *A12, double *A22, int engine) {
  if (engine < 0) engine = lu_update_engine<double>(c, m, n, k);
  if (engine == 1)
    return dgemm_emulated(0, 0, m, n, k, -1.0, A21, c.lda, A12, c.lda, 1.0, A22, c.lda, 0, c.s);
  gemm_minus<double>(m, n, k, A21, c.lda, A12, c.lda, A22, c.lda, c.s);
  return GB_SUCCESS;
}
template <>
int lu_update<float>(LuCtx<float> &c, int64_t m, int64_t n, int64_t k, const float *A21,
                     const float *A12, float *A22, int engine) {
  if (engine < 0) engine = lu_update_engine<float>(c, m, n, k);
  if (engine == 1)
    return sgemm_tc(0, 0, m, n, k, -1.0f, A21, c.lda, A12, c.lda, 1.0f, A22, c.lda, c.s);
  launch_sgemm_fp32(0, 0, m, n, k, -1.0f, A21, c.lda, A12, c.lda, 1.0f, A22, c.lda, c.s);
  return check_cuda(cudaGetLastError(), "sgemm launch");
}

// L11^-1 A12 of a blocked LU step.  With the emulated-FP64 updates and a
// block wider than 128 the triangle is solved in two halves on the FP64 pipe
// (lu_trsm) coupled by one emulated GEMM, B2 -= L21 X1, which halves the FP64
// work (the single-launch solve ran at ~1/4 of the FP64 pipe over the whole
// factorisation).  The form does not depend on the number of columns, and
// the coupling's default form (digit slices at this depth) gives every
// element from its own row and column only.
template <typename T>
int lu_trsm_block(const LuCtx<T> &c, int64_t n1, int64_t w, const T *L, int64_t ldl, T *B,
                  int64_t ldb, cudaStream_t s) {
  if constexpr (sizeof(T) == 8) {
    if (c.gemm_mode == 1 && n1 > 128 && w > 0) {
      const int64_t h = n1 / 2;
      int st;
      if ((st = lu_trsm<T>(h, w, L, ldl, B, ldb, s))) return st;
      if ((st = dgemm_emulated(0, 0, n1 - h, w, h, -1.0, L + h, ldl, B, ldb, 1.0, B + h, ldb, 0,
                               s)))
        return st;
      return lu_trsm<T>(n1 - h, w, L + h + h * ldl, ldl, B + h, ldb, s);
    }
  }
  return lu_trsm<T>(n1, w, L, ldl, B, ldb, s);
}

template <typename T>
int lu_panel_factor(LuCtx<T> &c, int64_t r0, int64_t m, int n) {
  ProfileScope prof("lu_panel", c.s);
  T *P = c.A + r0 + r0 * c.lda;
  if (c.use_cluster) {
    ProfileScope pc("lu_panel_cluster", c.s);
    const int st = launch_cluster_panel<T>(m, n, P, c.lda, c.ipiv + r0, r0, c.info, c.status,
                                           c.s);
    if (st != 1) return st;
  }
  GB_CUDA(cudaMemsetAsync(c.bar, 0, 2 * sizeof(unsigned), c.s));
  const int64_t b1 = (m + PANEL_THREADS - 1) / PANEL_THREADS;
  const int64_t b2 = (m + 2 * PANEL_THREADS - 1) / (2 * PANEL_THREADS);
  if (b1 <= c.lim1)
    return launch_panel<T, 1>(m, n, P, c.lda, c.ipiv + r0, r0, c.info, c.slots, c.bar, c.status,
                              (unsigned)b1, c.s);
  if (b2 <= c.lim2)
    return launch_panel<T, 2>(m, n, P, c.lda, c.ipiv + r0, r0, c.info, c.slots, c.bar, c.status,
                              (unsigned)b2, c.s);
  return set_error(GB_ERR_UNSUPPORTED, "getrf: %lld rows exceed the panel kernel limit",
                   (long long)m);
}

// Factor the leaf panel (columns r0 .. r0+n-1, rows r0 ..) and apply its row
// interchanges to the other columns of the outer block at once.  The
// reference's recursion applies them level by level -- to the right half
// before its TRSM, and to the left half after the right half is factored
// (getrf_single.c's recursive call) -- but between the panel and each of
// those points nothing reads or writes rows >= r0 of the columns concerned,
// so applying them earlier leaves every value where the reference puts it:
// one launch per panel instead of two per recursion level.  The same holds
// for the columns outside the outer block (the reference's LASWP before the
// block's TRSM and on the finished columns to the left), so for a matrix
// small enough that streaming all of it per panel stays cheap, the panel's
// interchanges reach every column; for larger ones they reach the outer
// block only and lu_blocked applies the block's interchanges to the other
// columns in two wide passes, which keeps the panel's data in L2.
template <typename T>
int lu_panel(LuCtx<T> &c, int64_t r0, int64_t m, int n) {
  int st = lu_panel_factor<T>(c, r0, m, n);
  if (st) return st;
  const int64_t npiv = m < n ? m : n;
  const int64_t width = c.blk1 - c.blk0;
  if (width <= n || npiv <= 0) return GB_SUCCESS;
  ProfileScope prof("lu_laswp", c.s);
  return launch_laswp_fused<T>(width - n, c.A + c.blk0 * c.lda, c.lda, r0 + 1, r0 + npiv, c.ipiv,
                               1, c.s, r0 - c.blk0, n);
}

// Factor the m x n block whose top-left corner is the diagonal entry (r0, r0); n <= m.
template <typename T>
int lu_rec(LuCtx<T> &c, int64_t r0, int64_t m, int64_t n) {
  // leaves of 32 columns, or 16 where a 32-column panel of m rows is too
  // tall for one cluster but a 16-column one fits (FP32)
  const int64_t leaf = c.use_cluster ? lu_leaf_width<T>(m) : PANEL_NB;
  if (n <= leaf) return lu_panel<T>(c, r0, m, (int)n);
  int64_t n1 = (n / 2) / leaf * leaf;
  if (n1 < leaf) n1 = leaf;
  const int64_t lda = c.lda;
  int st;
  // the left half's interchanges reach the right half inside lu_panel
  if ((st = lu_rec<T>(c, r0, m, n1))) return st;
  T *L11 = c.A + r0 + r0 * lda;
  T *A12 = c.A + r0 + (r0 + n1) * lda;
  {
    ProfileScope prof("lu_trsm", c.s);
    if ((st = lu_trsm<T>(n1, n - n1, L11, lda, A12, lda, c.s))) return st;
  }
  if (m > n1) {
    {
      ProfileScope prof("lu_gemm", c.s);
      if ((st = lu_update<T>(c, m - n1, n - n1, n1, L11 + n1, A12, A12 + n1))) return st;
    }
    if ((st = lu_rec<T>(c, r0 + n1, m - n1, n - n1))) return st;
  }
  return GB_SUCCESS;
}

// Outer right-looking loop over LU_OUTER_NB-wide block columns, each block
// factored recursively -- the structure of getrf_single.c:80-177 (blocking =
// min(mn/2, GEMM_Q), recursive call on the panel, LASWP + TRSM + GEMM on the
// trailing columns, later interchanges applied to the columns on the left).
constexpr int64_t LU_OUTER_NB = 256;
// With the emulated-FP64 updates and min(m, n) >= 16384 the block columns
// are twice as wide: the trailing updates then have depth 512 and take the
// modular scheme (14 residue products instead of 28 digit-slice products at
// depth 256, and half as many round trips of their planes through HBM).
// Measured: 16384^2 340 -> 319 ms; at 8192^2 the wider panels' inner solves
// cost more than that saves (94.6 -> 97.7 ms), so smaller matrices keep 256.
constexpr int64_t LU_OUTER_NB_EMULATED = 512;
static_assert(LU_OUTER_NB_EMULATED <= LASWP_FUSED_MAX, "a block's interchanges fit one fused LASWP");
template <typename T>
int64_t lu_outer_nb(const LuCtx<T> &c, int64_t mn) {
  return sizeof(T) == 8 && c.gemm_mode == 1 && mn >= 16384 ? LU_OUTER_NB_EMULATED : LU_OUTER_NB;
}

template <typename T>
int lu_blocked(LuCtx<T> &c, int64_t m, int64_t mn, int64_t n) {
  const int64_t lda = c.lda;
  int st;
  // measured on GB300 (FP32 LU): per-panel interchanges over the whole
  // width win at 8192^2 (268 MB), lose from 16384^2 (1 GB) on
  const bool whole = (double)c.nrows * (double)c.ncols * sizeof(T) <= 512.0 * 1024 * 1024;
  const int64_t onb = lu_outer_nb<T>(c, mn);
  for (int64_t j0 = 0; j0 < mn; j0 += onb) {
    const int64_t jb = (mn - j0) < onb ? (mn - j0) : onb;
    c.blk0 = whole ? 0 : j0;
    c.blk1 = whole ? c.ncols : j0 + jb;
    if ((st = lu_rec<T>(c, j0, m - j0, jb))) return st;
    // the block's interchanges (at most LASWP_FUSED_MAX) on the
    // trailing columns, then on the finished columns to the left
    const int64_t npiv = (m - j0) < jb ? (m - j0) : jb;
    if (!whole && j0 + jb < n) {
      ProfileScope prof("lu_laswp_right", c.s);
      if ((st = launch_laswp_fused<T>(n - j0 - jb, c.A + (j0 + jb) * lda, lda, j0 + 1,
                                      j0 + npiv, c.ipiv, 1, c.s)))
        return st;
    }
    if (!whole && j0 > 0) {
      ProfileScope prof("lu_laswp_left", c.s);
      if ((st = launch_laswp_fused<T>(j0, c.A, lda, j0 + 1, j0 + npiv, c.ipiv, 1, c.s)))
        return st;
    }
    T *L11 = c.A + j0 + j0 * lda;
    if (j0 + jb < n) {
      T *A12 = c.A + j0 + (j0 + jb) * lda;
      {
        ProfileScope prof("lu_trsm", c.s);
        if ((st = lu_trsm_block<T>(c, jb, n - j0 - jb, L11, lda, A12, lda, c.s))) return st;
      }
      if (j0 + jb < m) {
        ProfileScope prof("lu_gemm", c.s);
        if ((st = lu_update<T>(c, m - j0 - jb, n - j0 - jb, jb, L11 + jb, A12, A12 + jb)))
          return st;
      }
    }
  }
  return GB_SUCCESS;
}

// Right-looking blocked LU with a look-ahead of one block (the structure of
// lapack/getrf/getrf_parallel.c, where the thread that owns the next panel
// factors it as soon as its columns are updated, inner_advanced_thread, while
// the others finish the trailing update).  Block J+1's columns (the "slab")
// get block J's interchanges, triangular solve and update first, on the main
// stream; then block J+1 is factored on the highest-priority panel stream
// while the main stream applies block J's interchanges, solve and update to
// the remaining columns and its interchanges to the finished columns on the
// left.  Persistent GEMM kernels on the main stream leave SMs free for the
// panel meanwhile.  Every element sees exactly the operations of lu_blocked
// in the same order, so the factors and pivots are the same; the panels'
// interchanges reach their own block only, the rest being applied by the
// main stream once no kernel reads those rows.
//   main:   ... G(J-1, rest) | wait P(J) | X,T,G(J, slab) -> | X,T,G(J, rest), X(J, left) | ...
//   panel:  P(J) ------------------------------------------ | wait | P(J+1) -------------- |
template <typename T>
int lu_blocked_lookahead(LuCtx<T> &c, int64_t m, int64_t mn, int64_t n) {
  const int64_t lda = c.lda;
  cudaStream_t s = c.s, p = nullptr;
  cudaEvent_t to_panel = nullptr, to_main = nullptr;
  int st = lookahead_streams(&p, &to_panel, &to_main);
  if (st) return st;
  LuCtx<T> cp = c;  // the panel stream's context
  cp.s = p;
  const int64_t nb = LU_OUTER_NB;
  auto block_w = [&](int64_t j0) { return (mn - j0) < nb ? (mn - j0) : nb; };
  auto panel = [&](int64_t j0) -> int {
    cp.blk0 = j0;
    cp.blk1 = j0 + block_w(j0);
    int r = lu_rec<T>(cp, j0, m - j0, block_w(j0));
    if (r) return r;
    GB_CUDA(cudaEventRecord(to_main, p));
    return GB_SUCCESS;
  };
  // the panel stream starts after the work already queued on the main stream
  GB_CUDA(cudaEventRecord(to_panel, s));
  GB_CUDA(cudaStreamWaitEvent(p, to_panel, 0));
  if ((st = panel(0))) return st;
  // SMs the persistent GEMMs leave to the panel: one FP64/FP32 panel cluster
  const int reserve = 16;
  for (int64_t j0 = 0; j0 < mn; j0 += nb) {
    const int64_t jb = block_w(j0);
    const int64_t npiv = (m - j0) < jb ? (m - j0) : jb;
    const int64_t c0 = j0 + jb;                       // first trailing column
    const int64_t wslab = c0 < mn ? block_w(c0) : 0;  // the next block's columns
    GB_CUDA(cudaStreamWaitEvent(s, to_main, 0));      // block J is factored
    T *L11 = c.A + j0 + j0 * lda;
    // one engine for every column piece: the one the whole update would use
    const int engine = lu_update_engine<T>(c, m - c0, n - c0, jb);
    // block J's interchanges, solve and update on columns [a, a + w)
    auto update = [&](int64_t a, int64_t w) -> int {
      if (w <= 0) return GB_SUCCESS;
      int r;
      {
        ProfileScope prof("lu_laswp_right", s);
        if ((r = launch_laswp_fused<T>(w, c.A + a * lda, lda, j0 + 1, j0 + npiv, c.ipiv, 1, s)))
          return r;
      }
      T *A12 = c.A + j0 + a * lda;
      {
        ProfileScope prof("lu_trsm", s);
        if ((r = lu_trsm<T>(jb, w, L11, lda, A12, lda, s))) return r;
      }
      if (c0 < m) {
        ProfileScope prof("lu_gemm", s);
        if ((r = lu_update<T>(c, m - c0, w, jb, L11 + jb, A12, A12 + jb, engine))) return r;
      }
      return GB_SUCCESS;
    };
    if ((st = update(c0, wslab))) return st;
    if (wslab > 0) {
      GB_CUDA(cudaEventRecord(to_panel, s));
      GB_CUDA(cudaStreamWaitEvent(p, to_panel, 0));
      if ((st = panel(c0))) return st;
    }
    {
      SmReserve keep(reserve);
      if ((st = update(c0 + wslab, n - c0 - wslab))) return st;
    }
    if (j0 > 0) {
      ProfileScope prof("lu_laswp_left", s);
      if ((st = launch_laswp_fused<T>(j0, c.A, lda, j0 + 1, j0 + npiv, c.ipiv, 1, s))) return st;
    }
  }
  return GB_SUCCESS;
}

template <typename T>
int getrf_device_mode(int64_t m, int64_t n, T *A, int64_t lda, int *ipiv, int *info,
                      int gemm_mode, cudaStream_t s) {
  GB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
  const int64_t mn = m < n ? m : n;
  if (mn <= 0) return GB_SUCCESS;
  LuCtx<T> c;
  c.lim1 = coop_limit<T, 1>();
  c.lim2 = coop_limit<T, 2>();
  const int64_t maxblk = c.lim1 > c.lim2 ? c.lim1 : c.lim2;
  const size_t slot_elems = 2 * (size_t)maxblk * (PANEL_NB + 2) + 2 * PANEL_NB;
  Scratch ws(slot_elems * sizeof(T) + 256, s);
  if (!ws.p) return GB_ERR_ALLOC;
  c.A = A;
  c.lda = lda;
  c.ipiv = ipiv;
  c.info = info;
  c.slots = ws.as<T>();
  c.bar = reinterpret_cast<unsigned *>(reinterpret_cast<char *>(ws.p) +
                                       ((slot_elems * sizeof(T) + 127) & ~size_t(127)));
  c.status = ctx().d_status;
  c.gemm_mode = gemm_mode;
  c.nrows = m;
  c.ncols = n;
  c.s = s;
  // the outer loop already covers the columns right of the square part.
  // With two or more blocks and trailing updates on the FMA units, the next
  // panel is factored ahead (GB_LU_LOOKAHEAD=0 turns that off).  Not with the
  // tensor-core updates: their persistent kernels hold one CTA on every SM
  // (less the reserve) for the whole update, the panel's 16-CTA cluster then
  // finds no GPC with 16 free SMs and waits for the update anyway (measured:
  // FP32 LU 8192^2 24.9 -> 26.7 ms with look-ahead, 32768^2 panel time
  // 142 -> 266 ms), while the FMA kernels' CTAs retire and let it in (FP64
  // LU 8192^2 404 -> 361 ms).
  const bool ahead = mn > LU_OUTER_NB && config().lu_lookahead &&
                     lu_update_engine<T>(c, m - LU_OUTER_NB, n - LU_OUTER_NB, LU_OUTER_NB) == 0;
  int st = ahead ? lu_blocked_lookahead<T>(c, m, mn, n) : lu_blocked<T>(c, m, mn, n);
  if (st) return st;
  return check_cuda(cudaGetLastError(), "getrf");
}

template <typename T>
int getrf_device(int64_t m, int64_t n, T *A, int64_t lda, int *ipiv, int *info,
                 cudaStream_t s) {
  return getrf_device_mode<T>(m, n, A, lda, ipiv, info, 0, s);
}

template int getrf_device_mode<double>(int64_t, int64_t, double *, int64_t, int *, int *, int,
                                       cudaStream_t);

// ---------------------------------------------------------------------------
// LU without device allocation.
//
// Some callers cannot let a library allocate device memory: an application
// that hands every byte of HBM to its own arena or pool and forbids other
// allocations, a service that must stay inside a fixed memory budget for its
// whole life, or a caller that cannot afford the implicit synchronisation and
// latency of cudaMalloc/cudaFree in its loop.  For them the LU entry point
// below keeps the only scratch it needs -- the panel factorisation's
// parity-buffered candidate rows, its grid-barrier words and a status word --
// in this file-scope device array, so it makes no allocation at all.  The
// array is part of the loaded module: every GPU that uses the library holds
// these bytes until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr int NOALLOC_MAX_BLOCKS = 1024;  // cooperative panel blocks served
constexpr size_t NOALLOC_SLOT_BYTES =
    (2 * (size_t)NOALLOC_MAX_BLOCKS * (PANEL_NB + 2) + 2 * PANEL_NB) * sizeof(double);
constexpr size_t NOALLOC_SCRATCH_BYTES = 1u << 20;  // 1 MiB
static_assert(NOALLOC_SLOT_BYTES + 256 <= NOALLOC_SCRATCH_BYTES, "scratch too small");
// Rows the panel kernel can cover with the blocks above (two rows per thread).
constexpr int64_t NOALLOC_MAX_ROWS = (int64_t)NOALLOC_MAX_BLOCKS * 2 * PANEL_THREADS;

static __device__ __align__(256) unsigned char g_lu_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_lu_scratch per device, resolved once per device with
// that device current (host code must not use the symbol itself as an address).
std::mutex g_lu_scratch_mu;
void *g_lu_scratch_addr[64] = {nullptr};

int lu_scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return check_cuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return set_error(GB_ERR_UNSUPPORTED, "device index %d", dev);
  std::lock_guard<std::mutex> lk(g_lu_scratch_mu);
  if (!g_lu_scratch_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_lu_scratch);
    if (e != cudaSuccess) return check_cuda(e, "cudaGetSymbolAddress(g_lu_scratch)");
    g_lu_scratch_addr[dev] = p;
  }
  *out = g_lu_scratch_addr[dev];
  return GB_SUCCESS;
}

// Rows one panel can have on this device with the scratch above: the
// cluster panel (no slots) or the cooperative panel, whose grid is capped
// both by co-residency and by the NOALLOC_MAX_BLOCKS candidate slots.
int64_t noalloc_row_limit() {
  const ClusterPanel<double> caps = cluster_panel_caps<double>();
  const int64_t cl = caps.max_cs >= 2 ? (int64_t)caps.max_cs * CPANEL_THREADS * caps.lmax : 0;
  const int64_t b1 = coop_limit<double, 1>() < NOALLOC_MAX_BLOCKS ? coop_limit<double, 1>()
                                                                   : NOALLOC_MAX_BLOCKS;
  const int64_t b2 = coop_limit<double, 2>() < NOALLOC_MAX_BLOCKS ? coop_limit<double, 2>()
                                                                   : NOALLOC_MAX_BLOCKS;
  int64_t lim = cl;
  if (b1 * PANEL_THREADS > lim) lim = b1 * PANEL_THREADS;
  if (b2 * 2 * PANEL_THREADS > lim) lim = b2 * 2 * PANEL_THREADS;
  return lim;
}

// After the factorisation: a panel whose bounded grid barrier gave up left
// its status in the shared array, which no other call reads; report it
// through the caller's info word instead.
__global__ void noalloc_status_to_info_kernel(const int *__restrict__ status,
                                              int *__restrict__ info) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && status[0] != 0) *info = GB_INFO_WAIT_EXPIRED;
}

}  // namespace

}  // namespace gb

extern "C" int gb_dgetrf_noalloc_dev(int64_t m, int64_t n, double *A, int64_t lda, int *ipiv,
                                     int *info, void *stream) {
  using namespace gb;
  int code = 0;
  if (lda < (m > 1 ? m : 1)) code = 4;
  if (n < 0) code = 2;
  if (m < 0) code = 1;
  if (code) {
    call_xerbla("DGETRF", code);
    return GB_ERR_INVALID_VALUE;
  }
  if (m > NOALLOC_MAX_ROWS)
    return set_error(GB_ERR_UNSUPPORTED,
                     "gb_dgetrf_noalloc_dev: m = %lld exceeds the %lld rows its fixed scratch "
                     "serves",
                     (long long)m, (long long)NOALLOC_MAX_ROWS);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  void *base = nullptr;
  int st = lu_scratch_address(&base);
  if (st) return st;
  const int64_t mn = m < n ? m : n;
  if (mn > 0) {
    // the first panel has all m rows: refuse before any work is queued
    const int64_t lim = noalloc_row_limit();
    if (m > lim)
      return set_error(GB_ERR_UNSUPPORTED,
                       "gb_dgetrf_noalloc_dev: m = %lld exceeds the %lld rows one panel can "
                       "have on this device with the fixed scratch",
                       (long long)m, (long long)lim);
  }
  GB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
  if (mn <= 0) return GB_SUCCESS;
  LuCtx<double> c;
  c.lim1 = coop_limit<double, 1>();
  c.lim2 = coop_limit<double, 2>();
  if (c.lim1 > NOALLOC_MAX_BLOCKS) c.lim1 = NOALLOC_MAX_BLOCKS;
  if (c.lim2 > NOALLOC_MAX_BLOCKS) c.lim2 = NOALLOC_MAX_BLOCKS;
  char *b = reinterpret_cast<char *>(base);
  c.A = A;
  c.lda = lda;
  c.ipiv = ipiv;
  c.info = info;
  c.slots = reinterpret_cast<double *>(b);
  c.bar = reinterpret_cast<unsigned *>(b + ((NOALLOC_SLOT_BYTES + 127) & ~size_t(127)));
  c.status = reinterpret_cast<int *>(c.bar + 32);
  c.gemm_mode = 0;  // native FP64 trailing updates: no scratch anywhere below
  c.nrows = m;      // the panels' interchanges use the fused kernel: no scratch either
  c.ncols = n;
  c.s = s;
  // the shared array keeps the previous call's contents: clear the words that
  // must start at zero (barrier counters are cleared again before every panel)
  GB_CUDA(cudaMemsetAsync(c.bar, 0, 32 * sizeof(unsigned) + 4 * sizeof(int), s));
  if ((st = lu_blocked<double>(c, m, mn, n))) return st;
  { noalloc_status_to_info_kernel<<<1, 32, 0, s>>>(c.status, info); count_launch(); }
  return check_cuda(cudaGetLastError(), "gb_dgetrf_noalloc_dev");
}

namespace gb {

// lapack/getrs/getrs_single.c:42-68.  The interchanges of the solve are
// applied as one gather through the final permutation.
template <typename T>
int getrs_device(int trans, int64_t n, int64_t nrhs, const T *A, int64_t lda, const int *ipiv,
                 T *B, int64_t ldb, cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return GB_SUCCESS;
  Scratch ws(n * sizeof(int) + (size_t)n * nrhs * sizeof(T) + 256, s);
  if (!ws.p) return GB_ERR_ALLOC;
  int *perm = ws.as<int>();
  T *tmp = reinterpret_cast<T *>(reinterpret_cast<char *>(ws.p) +
                                 ((n * sizeof(int) + 127) & ~size_t(127)));
  { pivots_to_perm_kernel<<<1, 1, 0, s>>>(n, ipiv, perm); count_launch(); }
  const int64_t total = n * nrhs;
  const unsigned grid = (unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  int st;
  if (!trans) {
    { permute_rows_kernel<T><<<grid, 256, 0, s>>>(n, nrhs, perm, B, ldb, tmp, n, 0); count_launch(); }
    GB_CUDA(cudaMemcpy2DAsync(B, ldb * sizeof(T), tmp, n * sizeof(T), n * sizeof(T), nrhs,
                              cudaMemcpyDeviceToDevice, s));
    if ((st = trsm_any<T>(0, 1, 0, 0, n, nrhs, A, lda, B, ldb, s))) return st;
    if ((st = trsm_any<T>(0, 0, 0, 1, n, nrhs, A, lda, B, ldb, s))) return st;
  } else {
    if ((st = trsm_any<T>(0, 0, 1, 1, n, nrhs, A, lda, B, ldb, s))) return st;
    if ((st = trsm_any<T>(0, 1, 1, 0, n, nrhs, A, lda, B, ldb, s))) return st;
    { permute_rows_kernel<T><<<grid, 256, 0, s>>>(n, nrhs, perm, B, ldb, tmp, n, 1); count_launch(); }
    GB_CUDA(cudaMemcpy2DAsync(B, ldb * sizeof(T), tmp, n * sizeof(T), n * sizeof(T), nrhs,
                              cudaMemcpyDeviceToDevice, s));
  }
  return check_cuda(cudaGetLastError(), "getrs");
}

// Block columns of the blocked Cholesky (potrf_device_t below).
constexpr int64_t POTRF_NB = 256;

template <typename T>
int trsm_skip(int side, int uplo, int trans, int unit, int64_t m, int64_t n, const T *A,
              int64_t lda, T *B, int64_t ldb, cudaStream_t s, const int *skip);
template <>
int trsm_skip<double>(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                      const double *A, int64_t lda, double *B, int64_t ldb, cudaStream_t s,
                      const int *skip) {
  return dtrsm_device_skip(side, uplo, trans, unit, m, n, 1.0, A, lda, B, ldb, s, skip);
}
template <>
int trsm_skip<float>(int side, int uplo, int trans, int unit, int64_t m, int64_t n,
                     const float *A, int64_t lda, float *B, int64_t ldb, cudaStream_t s,
                     const int *skip) {
  return strsm_device_skip(side, uplo, trans, unit, m, n, 1.0f, A, lda, B, ldb, s, skip);
}
template <typename T>
int syrk_skip(int uplo, int trans, int64_t n, int64_t k, const T *A, int64_t lda, T *C,
              int64_t ldc, cudaStream_t s, const int *skip);
template <>
int syrk_skip<double>(int uplo, int trans, int64_t n, int64_t k, const double *A, int64_t lda,
                      double *C, int64_t ldc, cudaStream_t s, const int *skip) {
  return dsyrk_device_skip(uplo, trans, n, k, -1.0, A, lda, 1.0, C, ldc, s, skip);
}
template <>
int syrk_skip<float>(int uplo, int trans, int64_t n, int64_t k, const float *A, int64_t lda,
                     float *C, int64_t ldc, cudaStream_t s, const int *skip) {
  return ssyrk_device_skip(uplo, trans, n, k, -1.0f, A, lda, 1.0f, C, ldc, s, skip);
}

template <typename T>
static int potrf_diag_block(bool upper, int64_t nb, T *D, int64_t lda, int *info, int64_t off,
                            cudaStream_t s) {
  for (int64_t j0 = 0; j0 < nb; j0 += PANEL_NB) {
    const int jb = (int)((nb - j0) < PANEL_NB ? (nb - j0) : PANEL_NB);
    T *E = D + j0 + j0 * lda;
    { potf2_kernel<T><<<1, 256, 0, s>>>(upper ? 1 : 0, jb, E, lda, info, off + j0); count_launch(); }
    const int64_t rest = nb - j0 - jb;
    if (rest <= 0) continue;
    int st;
    if (!upper) {
      T *P = E + jb;
      if ((st = trsm_skip<T>(1, 1, 1, 1, rest, jb, E, lda, P, lda, s, info))) return st;
      if ((st = syrk_skip<T>(1, 0, rest, jb, P, lda, P + jb * lda, lda, s, info))) return st;
    } else {
      T *P = E + jb * lda;
      if ((st = trsm_skip<T>(0, 0, 1, 1, jb, rest, E, lda, P, lda, s, info))) return st;
      if ((st = syrk_skip<T>(0, 1, rest, jb, P, lda, P + jb, lda, s, info))) return st;
    }
  }
  return GB_SUCCESS;
}

// Trailing update C -= P P^T (lower) or P^T P (upper) of a 256-wide step:
// FP64 native or emulated (gemm_mode 1); FP32 on the tensor cores when large.
static int potrf_trailing(bool upper, int64_t rest, int64_t jb, const double *P, int64_t lda,
                          double *C, int *info, int gemm_mode, cudaStream_t s) {
  if (gemm_mode == 1 && rest >= 256 && jb >= 64)
    return upper ? dgemm_emulated(1, 0, rest, rest, jb, -1.0, P, lda, P, lda, 1.0, C, lda, 0, s, 2,
                                  info)
                 : dgemm_emulated(0, 1, rest, rest, jb, -1.0, P, lda, P, lda, 1.0, C, lda, 0, s, 1,
                                  info);
  return syrk_skip<double>(upper ? 0 : 1, upper ? 1 : 0, rest, jb, P, lda, C, lda, s, info);
}
static int potrf_trailing(bool upper, int64_t rest, int64_t jb, const float *P, int64_t lda,
                          float *C, int *info, int, cudaStream_t s) {
  const int mode = gb_get_sgemm_mode();
  if (mode == GB_SGEMM_TENSOR || (mode == GB_SGEMM_AUTO && rest >= 1024 && jb >= 64))
    return upper ? sgemm_tc(1, 0, rest, rest, jb, -1.0f, P, lda, P, lda, 1.0f, C, lda, s, 2, info)
                 : sgemm_tc(0, 1, rest, rest, jb, -1.0f, P, lda, P, lda, 1.0f, C, lda, s, 1, info);
  return syrk_skip<float>(upper ? 0 : 1, upper ? 1 : 0, rest, jb, P, lda, C, lda, s, info);
}

// Inverse of a lower triangle of at most 256 rows, by recursive doubling:
// the same identity as lapack/trtri/trtri_L_single.c:87-107 (whose block
// step forms W21 = -W22 L21 L11^-1 with TRMM and TRSM), evaluated as
// W21 = -W22 (L21 W11) over pairs of blocks of 32, 64 and 128.  Each level is
// one launch for every pair's T = L21 W11 and one for W21 = -W22 T, so the
// 256-wide inverse takes eight small launches; the native blocked TRSM on
// the identity took about fifteen (0.15 ms, launch- and latency-bound: the
// FP64 work is ~3 MFLOP).  L is the lower triangle of op(D) padded with the
// identity to npad (32 times a power of two): Lp(i, j) below.
__device__ __forceinline__ double trtri_lp(int jb, const double *__restrict__ D, int64_t lda,
                                           int tr, int i, int j) {
  if (i < jb && j < jb) return tr ? D[j + (int64_t)i * lda] : D[i + (int64_t)j * lda];
  return i == j ? 1.0 : 0.0;
}

// The 32 x 32 diagonal blocks of W = Lp^-1 (W zeroed beforehand): one warp
// per block, lane j the column j solve of Lp_bb w = e_j by the column sweep
// (w_c *= 1/l_cc, then w_r -= l_rc w_c for r > c).  The block is read column
// by column, a lane per row.
__global__ void __launch_bounds__(32)
trtri_diag32_kernel(int jb, const double *__restrict__ D, int64_t lda, int tr,
                    double *__restrict__ W, int64_t npad, const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double Ls[32][33];
  __shared__ double invd[32];
  const int lane = threadIdx.x, b0 = blockIdx.x * 32;
  double v[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) v[c] = lane >= c ? trtri_lp(jb, D, lda, tr, b0 + lane, b0 + c) : 0.0;
#pragma unroll
  for (int c = 0; c < 32; ++c) Ls[lane][c] = v[c];
  __syncwarp();
  invd[lane] = 1.0 / Ls[lane][lane];
  __syncwarp();
  double x[32];
#pragma unroll
  for (int r = 0; r < 32; ++r) x[r] = r == lane ? 1.0 : 0.0;
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    x[c] *= invd[c];
#pragma unroll
    for (int r = c + 1; r < 32; ++r) x[r] = fma(-Ls[r][c], x[c], x[r]);
  }
#pragma unroll
  for (int r = 0; r < 32; ++r) W[(b0 + r) + (int64_t)(b0 + lane) * npad] = x[r];
}

// One doubling level for block size sz <= 128: pair p covers rows/columns
// [2 sz p, 2 sz p + 2 sz).  FIRST: T_p = Lp21 W11; second: W21 = -W22 T_p.
// A CTA computes a 16 x 16 tile from its 16 rows of the left factor and 16
// columns of the right one, staged in shared memory by one coalesced round
// of loads; the sums run over all sz terms (the triangles' other entries
// are exact zeros), in four partial sums.
template <bool FIRST>
__global__ void __launch_bounds__(256)
trtri_level_kernel(int jb, const double *__restrict__ D, int64_t lda, int tr,
                   double *__restrict__ W, int64_t npad, int sz, double *__restrict__ T,
                   const int *__restrict__ skip) {
  if (skip && *skip) return;
  __shared__ double Xs[128][17];  // Xs[k][rr]: left factor, rows r0 + rr
  __shared__ double Ys[128][17];  // Ys[k][cc]: right factor, columns c0 + cc
  const int tid = threadIdx.x + 16 * threadIdx.y;
  const int r0 = blockIdx.x * 16, c0 = blockIdx.y * 16;
  const int o = 2 * sz * blockIdx.z;
  double *Tp = T + (int64_t)blockIdx.z * sz * sz;
  for (int e = tid; e < 16 * sz; e += 256) {
    const int rr = e & 15, k = e >> 4;  // 16 consecutive rows (or k) per group
    Xs[k][rr] = FIRST ? trtri_lp(jb, D, lda, tr, o + sz + r0 + rr, o + k)
                      : W[(o + sz + r0 + rr) + (int64_t)(o + sz + k) * npad];
  }
  for (int e = tid; e < 16 * sz; e += 256) {
    const int k = e % sz, cc = e / sz;
    Ys[k][cc] = FIRST ? W[(o + k) + (int64_t)(o + c0 + cc) * npad] : Tp[k + (int64_t)(c0 + cc) * sz];
  }
  __syncthreads();
  const int rr = threadIdx.x, cc = threadIdx.y;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  for (int k = 0; k < sz; k += 4) {  // sz is a multiple of 32
    a0 = fma(Xs[k][rr], Ys[k][cc], a0);
    a1 = fma(Xs[k + 1][rr], Ys[k + 1][cc], a1);
    a2 = fma(Xs[k + 2][rr], Ys[k + 2][cc], a2);
    a3 = fma(Xs[k + 3][rr], Ys[k + 3][cc], a3);
  }
  const double sum = (a0 + a1) + (a2 + a3);
  if (FIRST)
    Tp[(r0 + rr) + (int64_t)(c0 + cc) * sz] = sum;
  else
    W[(o + sz + r0 + rr) + (int64_t)(o + c0 + cc) * npad] = -sum;
}

// W (npad x npad, leading dimension npad) := the inverse of the lower
// triangle of op(D) (jb <= npad rows; op(D) = D, or D^T when tr), the
// identity beyond jb.  T: npad^2 / 4 doubles of scratch.
static int trtri_lower_fp64(int64_t jb, const double *D, int64_t lda, int tr, double *W,
                            int64_t npad, double *T, cudaStream_t s, const int *skip) {
  if (npad > 256) return set_error(GB_ERR_UNSUPPORTED, "trtri: triangle wider than 256");
  GB_CUDA(cudaMemsetAsync(W, 0, (size_t)npad * npad * sizeof(double), s));
  { trtri_diag32_kernel<<<(unsigned)(npad / 32), 32, 0, s>>>((int)jb, D, lda, tr, W, npad, skip); count_launch(); }
  for (int64_t sz = 32; sz < npad; sz *= 2) {
    const dim3 g((unsigned)(sz / 16), (unsigned)(sz / 16), (unsigned)(npad / (2 * sz)));
    { trtri_level_kernel<true><<<g, dim3(16, 16), 0, s>>>((int)jb, D, lda, tr, W, npad, (int)sz, T, skip); count_launch(); }
    { trtri_level_kernel<false><<<g, dim3(16, 16), 0, s>>>((int)jb, D, lda, tr, W, npad, (int)sz, T, skip); count_launch(); }
  }
  return check_cuda(cudaGetLastError(), "trtri");
}

// The panel solve of a 256-wide step: L21 = A21 L11^-T (lower) or
// U12 = U11^-T A12 (upper).  Native: one FP64 TRSM.  In the emulated-FP64
// mode the block's triangle is inverted once (native FP64, jb^3/3 flops, by
// trtri_lower_fp64) and the panel becomes one FP64-accurate GEMM on
// the tensor cores -- the native TRSM over the whole panel ran at the FP64
// pipe's rate (152 of 884 ms at n = 32768).  Steps after a failed pivot are
// skipped on the device (info), as in the native form.
static int potrf_panel_solve(bool upper, int64_t rest, int64_t jb, const double *D,
                             int64_t lda, double *P, int *info, int gemm_mode, cudaStream_t s) {
  if (gemm_mode == 1 && rest >= 256 && jb > POTRF_NB) {
    // a block wider than 256: blocked substitution over its 256-wide block
    // columns, each one's triangle inverted as below and the coupling with
    // the block columns before it applied as one emulated GEMM (depth 256 i)
    for (int64_t i0 = 0; i0 < jb; i0 += POTRF_NB) {
      const int64_t ib = (jb - i0) < POTRF_NB ? (jb - i0) : POTRF_NB;
      int st;
      if (upper) {
        double *Pi = P + i0;  // rows i0.. of the jb x rest panel
        if (i0 > 0) {
          ProfileScope prof("potrf_couple", s);
          if ((st = dgemm_emulated(1, 0, ib, rest, i0, -1.0, D + i0 * lda, lda, P, lda, 1.0, Pi,
                                   lda, 0, s, 0, info)))
            return st;
        }
        if ((st = potrf_panel_solve(true, rest, ib, D + i0 + i0 * lda, lda, Pi, info, gemm_mode,
                                    s)))
          return st;
      } else {
        double *Pi = P + i0 * lda;  // columns i0.. of the rest x jb panel
        if (i0 > 0) {
          ProfileScope prof("potrf_couple", s);
          if ((st = dgemm_emulated(0, 1, rest, ib, i0, -1.0, P, lda, D + i0, lda, 1.0, Pi, lda, 0,
                                   s, 0, info)))
            return st;
        }
        if ((st = potrf_panel_solve(false, rest, ib, D + i0 + i0 * lda, lda, Pi, info, gemm_mode,
                                    s)))
          return st;
      }
    }
    return GB_SUCCESS;
  }
  if (!(gemm_mode == 1 && rest >= 256 && jb >= 64))
    return upper ? trsm_skip<double>(0, 0, 1, 1, jb, rest, D, lda, P, lda, s, info)
                 : trsm_skip<double>(1, 1, 1, 1, rest, jb, D, lda, P, lda, s, info);
  int64_t npad = 32;
  while (npad < jb) npad *= 2;
  Scratch ws((size_t)(npad * npad + npad * npad / 4 + rest * jb) * sizeof(double), s);
  if (!ws.p) return GB_ERR_ALLOC;
  double *W = ws.as<double>(), *Tl = W + npad * npad, *T = Tl + npad * npad / 4;
  int st;
  {
    // W := the inverse of the block's lower triangle (L), or of the lower
    // triangle of D^T (U^T, whose inverse is U^-T): non-unit
    ProfileScope prof("potrf_inv", s);
    st = trtri_lower_fp64(jb, D, lda, upper ? 1 : 0, W, npad, Tl, s, info);
  }
  if (st) return st;
  ProfileScope prof("potrf_apply", s);
  if (upper) {  // P (jb x rest) := U^-T P = W P
    GB_CUDA(cudaMemcpy2DAsync(T, jb * 8, P, lda * 8, jb * 8, rest, cudaMemcpyDeviceToDevice, s));
    return dgemm_emulated(0, 0, jb, rest, jb, 1.0, W, npad, T, jb, 0.0, P, lda, 0, s, 0, info);
  }
  // P (rest x jb) := P L^-T = P W^T
  GB_CUDA(cudaMemcpy2DAsync(T, rest * 8, P, lda * 8, rest * 8, jb, cudaMemcpyDeviceToDevice, s));
  return dgemm_emulated(0, 1, rest, jb, jb, 1.0, T, rest, W, npad, 0.0, P, lda, 0, s, 0, info);
}
static int potrf_panel_solve(bool upper, int64_t rest, int64_t jb, const float *D, int64_t lda,
                             float *P, int *info, int, cudaStream_t s) {
  return upper ? trsm_skip<float>(0, 0, 1, 1, jb, rest, D, lda, P, lda, s, info)
               : trsm_skip<float>(1, 1, 1, 1, rest, jb, D, lda, P, lda, s, info);
}

// Cholesky, blocked like lapack/potrf/potrf_L_single.c / potrf_U_single.c:
// 256-wide block columns; the diagonal block is factored by 32-wide steps
// (potf2 + TRSM + SYRK inside the block); the panel below (right of) it is
// solved against the block's triangle (potrf_panel_solve), and the trailing
// matrix gets one rank-256 SYRK (see potrf_trailing).  Every step after a non-positive pivot
// is skipped on the device (info), so the matrix is left as it was at the
// failing column.  With emulated-FP64 updates (FP64, gemm_mode 1) the block
// columns are POTRF_NB_EMULATED wide and each diagonal block is itself
// factored by this routine with 256-wide blocks: every outer emulated panel
// solve and trailing update then has depth k = 2048, which amortises the
// residue planes' round trip through HBM over eight times the work and takes
// the modular scheme (k >= 512); measured at 32768: 1024-wide 359 ms,
// 2048-wide 332 ms, 4096-wide with 1024-wide inner blocks 350 ms.
// off: the global column of A(0,0) (for info).
constexpr int64_t POTRF_NB_EMULATED = 2048;
template <typename T>
int potrf_blocked(int uplo, int64_t n, T *A, int64_t lda, int *info, int gemm_mode,
                  cudaStream_t s, int64_t nb, int64_t off) {
  const bool upper = uplo == 0;
  for (int64_t j0 = 0; j0 < n; j0 += nb) {
    const int64_t jb = (n - j0) < nb ? (n - j0) : nb;
    T *D = A + j0 + j0 * lda;
    int st;
    {
      ProfileScope prof("potrf_diag", s);
      if (jb > POTRF_NB) {
        if ((st = potrf_blocked<T>(uplo, jb, D, lda, info, gemm_mode, s, POTRF_NB, off + j0)))
          return st;
      } else if ((st = potrf_diag_block<T>(upper, jb, D, lda, info, off + j0, s))) {
        return st;
      }
    }
    const int64_t rest = n - j0 - jb;
    if (rest <= 0) continue;
    T *P = upper ? A + j0 + (j0 + jb) * lda   // jb x rest
                 : A + (j0 + jb) + j0 * lda;  // rest x jb
    {
      ProfileScope prof("potrf_trsm", s);
      if ((st = potrf_panel_solve(upper, rest, jb, D, lda, P, info, gemm_mode, s))) return st;
    }
    {
      ProfileScope prof("potrf_update", s);
      st = upper ? potrf_trailing(true, rest, jb, P, lda, P + jb, info, gemm_mode, s)
                 : potrf_trailing(false, rest, jb, P, lda, P + jb * lda, info, gemm_mode, s);
    }
    if (st) return st;
  }
  return check_cuda(cudaGetLastError(), "potrf");
}

template <typename T>
int potrf_device_t(int uplo, int64_t n, T *A, int64_t lda, int *info, int gemm_mode,
                   cudaStream_t s) {
  GB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), s));
  const int64_t nb = (sizeof(T) == 8 && gemm_mode == 1) ? POTRF_NB_EMULATED : POTRF_NB;
  return potrf_blocked<T>(uplo, n, A, lda, info, gemm_mode, s, nb, 0);
}

int potrf_device(int uplo, int64_t n, double *A, int64_t lda, int *info, int gemm_mode,
                 cudaStream_t s) {
  return potrf_device_t<double>(uplo, n, A, lda, info, gemm_mode, s);
}

int spotrf_device(int uplo, int64_t n, float *A, int64_t lda, int *info, cudaStream_t s) {
  return potrf_device_t<float>(uplo, n, A, lda, info, 0, s);
}

// A X = B with A = L L^T (lower) or U^T U (upper): dpotrs.f:135-160.
int potrs_device(int uplo, int64_t n, int64_t nrhs, const double *A, int64_t lda, double *B,
                 int64_t ldb, cudaStream_t s) {
  int st;
  if (uplo == 1) {
    if ((st = dtrsm_device(0, 1, 0, 1, n, nrhs, 1.0, A, lda, B, ldb, s))) return st;
    return dtrsm_device(0, 1, 1, 1, n, nrhs, 1.0, A, lda, B, ldb, s);
  }
  if ((st = dtrsm_device(0, 0, 1, 1, n, nrhs, 1.0, A, lda, B, ldb, s))) return st;
  return dtrsm_device(0, 0, 0, 1, n, nrhs, 1.0, A, lda, B, ldb, s);
}

int pivots_to_perm(int64_t n, const int *ipiv, int *perm, cudaStream_t s) {
  { pivots_to_perm_kernel<<<1, 1, 0, s>>>(n, ipiv, perm); count_launch(); }
  return check_cuda(cudaGetLastError(), "pivots_to_perm");
}

template <typename T>
int apply_perm(int64_t n, int64_t ncol, const int *perm, const T *src, int64_t lds, T *dst,
               int64_t ldd, cudaStream_t s) {
  const int64_t total = n * ncol;
  const unsigned grid = (unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  { permute_rows_kernel<T><<<grid, 256, 0, s>>>(n, ncol, perm, src, lds, dst, ldd, 0); count_launch(); }
  return check_cuda(cudaGetLastError(), "apply_perm");
}
template int apply_perm<float>(int64_t, int64_t, const int *, const float *, int64_t, float *,
                               int64_t, cudaStream_t);
template int apply_perm<double>(int64_t, int64_t, const int *, const double *, int64_t,
                                double *, int64_t, cudaStream_t);

template int getrf_device<double>(int64_t, int64_t, double *, int64_t, int *, int *,
                                  cudaStream_t);
template int getrf_device<float>(int64_t, int64_t, float *, int64_t, int *, int *, cudaStream_t);
template int getrs_device<double>(int, int64_t, int64_t, const double *, int64_t, const int *,
                                  double *, int64_t, cudaStream_t);
template int getrs_device<float>(int, int64_t, int64_t, const float *, int64_t, const int *,
                                 float *, int64_t, cudaStream_t);
template int laswp_device<double>(int64_t, double *, int64_t, int64_t, int64_t, const int *,
                                  int64_t, cudaStream_t);
template int laswp_device<float>(int64_t, float *, int64_t, int64_t, int64_t, const int *,
                                 int64_t, cudaStream_t);

}  // namespace gb
