/*
 * oracle.c -- CPU restatement of OpenBLAS's level-3 + blocked-LAPACK hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the reference results the library is tested
 * against.  Loaded by the tests, the smoke check and bench.py's CPU-baseline
 * leg; never by the product library.
 *
 * Each function cites the OpenBLAS 0.3.28.dev source it restates.  The code
 * is written from those algorithms, not copied: the GotoBLAS packing/kernel
 * split is replaced by a plain cache-blocked loop nest with OpenMP threads,
 * which keeps the arithmetic contract (what is computed, pivot rules, info
 * codes, beta/alpha special cases) while using portable C.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;

void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

static inline int upc(char c) { return (c >= 'a' && c <= 'z') ? c - 32 : c; }
static inline int is_trans(char t) {
  t = (char)upc(t);
  return t == 'T' || t == 'C';
}

/* ------------------------------------------------------------------------ */
/* GEMM                                                                      */
/* ------------------------------------------------------------------------ */

/* Cache blocking of the oracle GEMM: C is cut into MCxNC tiles (one per
 * OpenMP task); each tile loops over KC-deep slabs whose operands are packed
 * into contiguous MRxKC / KCxNR micro-panels.  Plays the role of the Goto
 * js/ls/is loops of driver/level3/level3.c:288-408. */
#define ORC_MR 8
#define ORC_NR 4
#define ORC_MC 128
#define ORC_NC 128
#define ORC_KC 256

#define DEFINE_GEMM(NAME, T)                                                   \
  static void NAME##_beta(int m, int n, T beta, T *C, int ldc) {               \
    /* kernel/generic/gemm_beta.c:41-94: beta==0 stores zeros. */              \
    if (beta == (T)1) return;                                                  \
    for (int j = 0; j < n; ++j) {                                              \
      T *c = C + (size_t)j * ldc;                                              \
      if (beta == (T)0)                                                        \
        for (int i = 0; i < m; ++i) c[i] = (T)0;                               \
      else                                                                     \
        for (int i = 0; i < m; ++i) c[i] *= beta;                              \
    }                                                                          \
  }                                                                            \
  static void NAME##_tile(int ta, int tb, int i0, int mc, int j0, int nc,     \
                          int k, T alpha, const T *A, int lda, const T *B,     \
                          int ldb, T *C, int ldc, T *ap, T *bp) {              \
    for (int p0 = 0; p0 < k; p0 += ORC_KC) {                                   \
      int kc = k - p0 < ORC_KC ? k - p0 : ORC_KC;                              \
      /* pack op(A)[i0:i0+mc, p0:p0+kc] into MR-row panels, k-major */         \
      for (int ib = 0; ib < mc; ib += ORC_MR) {                                \
        T *dst = ap + (size_t)ib * kc;                                         \
        for (int p = 0; p < kc; ++p)                                           \
          for (int r = 0; r < ORC_MR; ++r) {                                   \
            int i = i0 + ib + r;                                               \
            T v = (T)0;                                                        \
            if (ib + r < mc)                                                   \
              v = ta ? A[(size_t)i * lda + p0 + p]                             \
                     : A[(size_t)(p0 + p) * lda + i];                          \
            dst[(size_t)p * ORC_MR + r] = v;                                   \
          }                                                                    \
      }                                                                        \
      /* pack op(B)[p0:p0+kc, j0:j0+nc] into NR-column panels */               \
      for (int jb = 0; jb < nc; jb += ORC_NR) {                                \
        T *dst = bp + (size_t)jb * kc;                                         \
        for (int p = 0; p < kc; ++p)                                           \
          for (int c = 0; c < ORC_NR; ++c) {                                   \
            int j = j0 + jb + c;                                               \
            T v = (T)0;                                                        \
            if (jb + c < nc)                                                   \
              v = tb ? B[(size_t)(p0 + p) * ldb + j]                           \
                     : B[(size_t)j * ldb + p0 + p];                            \
            dst[(size_t)p * ORC_NR + c] = v;                                   \
          }                                                                    \
      }                                                                        \
      for (int jb = 0; jb < nc; jb += ORC_NR) {                                \
        for (int ib = 0; ib < mc; ib += ORC_MR) {                              \
          const T *a = ap + (size_t)ib * kc;                                   \
          const T *b = bp + (size_t)jb * kc;                                   \
          T acc[ORC_NR][ORC_MR];                                               \
          for (int c = 0; c < ORC_NR; ++c)                                     \
            for (int r = 0; r < ORC_MR; ++r) acc[c][r] = (T)0;                 \
          for (int p = 0; p < kc; ++p) {                                       \
            const T *ar = a + (size_t)p * ORC_MR;                              \
            const T *br = b + (size_t)p * ORC_NR;                              \
            for (int c = 0; c < ORC_NR; ++c)                                   \
              for (int r = 0; r < ORC_MR; ++r) acc[c][r] += ar[r] * br[c];     \
          }                                                                    \
          int mr = mc - ib < ORC_MR ? mc - ib : ORC_MR;                        \
          int nr = nc - jb < ORC_NR ? nc - jb : ORC_NR;                        \
          for (int c = 0; c < nr; ++c) {                                       \
            T *cc = C + (size_t)(j0 + jb + c) * ldc + i0 + ib;                 \
            for (int r = 0; r < mr; ++r) cc[r] += alpha * acc[c][r];           \
          }                                                                    \
        }                                                                      \
      }                                                                        \
    }                                                                          \
  }                                                                            \
  void NAME(char transa, char transb, int m, int n, int k, T alpha,           \
            const T *A, int lda, const T *B, int ldb, T beta, T *C, int ldc) { \
    if (m <= 0 || n <= 0) return;                                              \
    int ta = is_trans(transa), tb = is_trans(transb);                          \
    NAME##_beta(m, n, beta, C, ldc);                                           \
    /* level3.c:252-259: nothing more when k==0 or alpha==0 */                 \
    if (k <= 0 || alpha == (T)0) return;                                       \
    int mt = (m + ORC_MC - 1) / ORC_MC, nt = (n + ORC_NC - 1) / ORC_NC;        \
    int ntiles = mt * nt;                                                      \
    int nthr = orc_get_threads();                                              \
    if ((double)m * n * k < 2e6) nthr = 1;                                     \
    _Pragma("omp parallel num_threads(nthr)") {                                \
      T *ap = (T *)malloc(sizeof(T) * (ORC_MC + ORC_MR) * ORC_KC);             \
      T *bp = (T *)malloc(sizeof(T) * (ORC_NC + ORC_NR) * ORC_KC);             \
      _Pragma("omp for schedule(dynamic, 1)") for (int t = 0; t < ntiles;      \
                                                   ++t) {                      \
        int it = t % mt, jt = t / mt;                                          \
        int i0 = it * ORC_MC, j0 = jt * ORC_NC;                                \
        int mc = m - i0 < ORC_MC ? m - i0 : ORC_MC;                            \
        int nc = n - j0 < ORC_NC ? n - j0 : ORC_NC;                            \
        NAME##_tile(ta, tb, i0, mc, j0, nc, k, alpha, A, lda, B, ldb, C, ldc,  \
                    ap, bp);                                                   \
      }                                                                        \
      free(ap);                                                                \
      free(bp);                                                                \
    }                                                                          \
  }

DEFINE_GEMM(orc_dgemm, double)
DEFINE_GEMM(orc_sgemm, float)

/* --- double-double reference ------------------------------------------- */
static inline void two_sum(double a, double b, double *s, double *e) {
  double x = a + b;
  double bb = x - a;
  *e = (a - (x - bb)) + (b - bb);
  *s = x;
}
static inline void dd_add_prod(double *hi, double *lo, double a, double b) {
  double p = a * b;
  double pe = fma(a, b, -p);
  double s, e;
  two_sum(*hi, p, &s, &e);
  e += *lo + pe;
  two_sum(s, e, hi, lo);
}

void orc_dgemm_dd(char transa, char transb, int m, int n, int k, double alpha,
                  const double *A, int lda, const double *B, int ldb,
                  double beta, double *C, int ldc) {
  if (m <= 0 || n <= 0) return;
  int ta = is_trans(transa), tb = is_trans(transb);
  int nthr = orc_get_threads();
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 4)
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < m; ++i) {
      double hi = 0.0, lo = 0.0;
      for (int p = 0; p < k; ++p) {
        double a = ta ? A[(size_t)i * lda + p] : A[(size_t)p * lda + i];
        double b = tb ? B[(size_t)p * ldb + j] : B[(size_t)j * ldb + p];
        dd_add_prod(&hi, &lo, a, b);
      }
      /* r = alpha*(hi+lo) + beta*c, still in double-double */
      double rh = 0.0, rl = 0.0;
      if (k > 0 && alpha != 0.0) {
        dd_add_prod(&rh, &rl, alpha, hi);
        dd_add_prod(&rh, &rl, alpha, lo);
      }
      double c = C[(size_t)j * ldc + i];
      if (beta != 0.0) dd_add_prod(&rh, &rl, beta, c);
      C[(size_t)j * ldc + i] = rh + rl;
    }
  }
}

void orc_dgemm_absbound(char transa, char transb, int m, int n, int k,
                        double alpha, const double *A, int lda, const double *B,
                        int ldb, double beta, const double *C, int ldc,
                        double *G, int ldg) {
  if (m <= 0 || n <= 0) return;
  int ta = is_trans(transa), tb = is_trans(transb);
  int nthr = orc_get_threads();
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 4)
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int p = 0; p < k; ++p) {
        double a = ta ? A[(size_t)i * lda + p] : A[(size_t)p * lda + i];
        double b = tb ? B[(size_t)p * ldb + j] : B[(size_t)j * ldb + p];
        s += fabs(a) * fabs(b);
      }
      G[(size_t)j * ldg + i] =
          fabs(alpha) * s + fabs(beta) * fabs(C[(size_t)j * ldc + i]);
    }
}

/* ------------------------------------------------------------------------ */
/* TRSM                                                                      */
/* ------------------------------------------------------------------------ */
/* Solves the triangular system column by column (Left) or row by row
 * (Right) after scaling B by alpha, as driver/level3/trsm_L.c:103-113 and
 * trsm_R.c do with GEMM_BETA.  The 8 side/trans x uplo cases reduce to a
 * forward or backward substitution on op(A). */
#define DEFINE_TRSM(NAME, T)                                                   \
  void NAME(char side, char uplo, char transa, char diag, int m, int n,       \
            T alpha, const T *A, int lda, T *B, int ldb) {                     \
    if (m <= 0 || n <= 0) return;                                              \
    int left = upc(side) == 'L';                                               \
    int lower = upc(uplo) == 'L';                                              \
    int tr = is_trans(transa);                                                 \
    int unit = upc(diag) == 'U';                                               \
    int nthr = orc_get_threads();                                              \
    if ((double)m * n * (left ? m : n) < 1e6) nthr = 1;                        \
    if (alpha != (T)1) {                                                       \
      for (int j = 0; j < n; ++j)                                              \
        for (int i = 0; i < m; ++i)                                            \
          B[(size_t)j * ldb + i] =                                             \
              alpha == (T)0 ? (T)0 : alpha * B[(size_t)j * ldb + i];           \
      if (alpha == (T)0) return;                                               \
    }                                                                          \
    /* effective lower-ness of op(A) */                                        \
    int eff_lower = lower ^ tr;                                                \
    if (left) {                                                                \
      /* op(A) X = B, each column independent */                               \
      _Pragma("omp parallel for num_threads(nthr) schedule(static)") for (     \
          int j = 0; j < n; ++j) {                                             \
        T *b = B + (size_t)j * ldb;                                            \
        if (!tr) {                                                             \
          if (eff_lower) {                                                     \
            for (int kk = 0; kk < m; ++kk) {                                   \
              if (b[kk] == (T)0) continue;                                     \
              if (!unit) b[kk] /= A[(size_t)kk * lda + kk];                    \
              T t = b[kk];                                                     \
              const T *a = A + (size_t)kk * lda;                               \
              for (int i = kk + 1; i < m; ++i) b[i] -= t * a[i];               \
            }                                                                  \
          } else {                                                             \
            for (int kk = m - 1; kk >= 0; --kk) {                              \
              if (b[kk] == (T)0) continue;                                     \
              if (!unit) b[kk] /= A[(size_t)kk * lda + kk];                    \
              T t = b[kk];                                                     \
              const T *a = A + (size_t)kk * lda;                               \
              for (int i = 0; i < kk; ++i) b[i] -= t * a[i];                   \
            }                                                                  \
          }                                                                    \
        } else {                                                               \
          /* op(A) = A^T: row i of op(A) is column i of A */                   \
          if (eff_lower) { /* A upper, forward */                              \
            for (int i = 0; i < m; ++i) {                                      \
              const T *a = A + (size_t)i * lda;                                \
              T t = b[i];                                                      \
              for (int p = 0; p < i; ++p) t -= a[p] * b[p];                    \
              if (!unit) t /= a[i];                                            \
              b[i] = t;                                                        \
            }                                                                  \
          } else { /* A lower, backward */                                     \
            for (int i = m - 1; i >= 0; --i) {                                 \
              const T *a = A + (size_t)i * lda;                                \
              T t = b[i];                                                      \
              for (int p = i + 1; p < m; ++p) t -= a[p] * b[p];                \
              if (!unit) t /= a[i];                                            \
              b[i] = t;                                                        \
            }                                                                  \
          }                                                                    \
        }                                                                      \
      }                                                                        \
    } else {                                                                   \
      /* X op(A) = B: column j of X depends on columns of X by op(A) */        \
      /* op(A)[p][j] = tr ? A[j][p] : A[p][j] */                               \
      int fwd = !eff_lower; /* upper op(A): X[:,j] uses X[:,p<j] */            \
      for (int jj = 0; jj < n; ++jj) {                                         \
        int j = fwd ? jj : n - 1 - jj;                                         \
        T *bj = B + (size_t)j * ldb;                                           \
        int p0 = fwd ? 0 : j + 1, p1 = fwd ? j : n;                            \
        for (int p = p0; p < p1; ++p) {                                        \
          T apj = tr ? A[(size_t)p * lda + j] : A[(size_t)j * lda + p];        \
          if (apj == (T)0) continue;                                           \
          const T *bp = B + (size_t)p * ldb;                                   \
          for (int i = 0; i < m; ++i) bj[i] -= apj * bp[i];                    \
        }                                                                      \
        if (!unit) {                                                           \
          T d = A[(size_t)j * lda + j];                                        \
          for (int i = 0; i < m; ++i) bj[i] /= d;                              \
        }                                                                      \
      }                                                                        \
    }                                                                          \
  }

DEFINE_TRSM(orc_dtrsm, double)
DEFINE_TRSM(orc_strsm, float)

/* ------------------------------------------------------------------------ */
/* SYRK                                                                      */
/* ------------------------------------------------------------------------ */
void orc_dsyrk(char uplo, char trans, int n, int k, double alpha,
               const double *A, int lda, double beta, double *C, int ldc) {
  if (n <= 0) return;
  int lower = upc(uplo) == 'L';
  int tr = is_trans(trans);
  /* syrk_k.c:52-105: triangular beta scaling first (beta==0 stores 0) */
  for (int j = 0; j < n; ++j) {
    int i0 = lower ? j : 0, i1 = lower ? n : j + 1;
    double *c = C + (size_t)j * ldc;
    if (beta == 0.0)
      for (int i = i0; i < i1; ++i) c[i] = 0.0;
    else if (beta != 1.0)
      for (int i = i0; i < i1; ++i) c[i] *= beta;
  }
  if (k <= 0 || alpha == 0.0) return;
  int nthr = orc_get_threads();
  if ((double)n * n * k < 2e6) nthr = 1;
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 8)
  for (int j = 0; j < n; ++j) {
    int i0 = lower ? j : 0, i1 = lower ? n : j + 1;
    double *c = C + (size_t)j * ldc;
    if (!tr) {
      /* C += alpha * A A^T : C[i][j] += sum_p A[i][p] A[j][p] */
      for (int p = 0; p < k; ++p) {
        double t = alpha * A[(size_t)p * lda + j];
        if (t == 0.0) continue;
        const double *a = A + (size_t)p * lda;
        for (int i = i0; i < i1; ++i) c[i] += t * a[i];
      }
    } else {
      /* C += alpha * A^T A : C[i][j] += sum_p A[p][i] A[p][j] */
      const double *aj = A + (size_t)j * lda;
      for (int i = i0; i < i1; ++i) {
        const double *ai = A + (size_t)i * lda;
        double s = 0.0;
        for (int p = 0; p < k; ++p) s += ai[p] * aj[p];
        c[i] += alpha * s;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* LASWP / GETF2 / GETRF / GETRS / GESV                                      */
/* ------------------------------------------------------------------------ */
#define DEFINE_LU(PFX, T, TMIN, GEMM, TRSM)                                    \
  void PFX##laswp(int n, T *A, int lda, int k1, int k2, const int *ipiv,      \
                  int incx) {                                                  \
    /* interface/lapack/laswp.c:55-110: incx==0 or n<=0 is a no-op; incx<0    \
     * walks the pivots backwards (laswp_k_1.c MINUS variant). */              \
    if (incx == 0 || n <= 0 || k2 < k1) return;                                \
    int cnt = k2 - k1 + 1;                                                     \
    for (int j = 0; j < n; ++j) {                                              \
      T *a = A + (size_t)j * lda;                                              \
      for (int t = 0; t < cnt; ++t) {                                          \
        int i = incx > 0 ? k1 + t : k2 - t;                     /* 1-based */  \
        int pidx = incx > 0 ? (k1 - 1) + t * incx                              \
                            : (k1 - 1) + (cnt - 1 - t) * (-incx);              \
        int ip = ipiv[pidx];                                                   \
        if (ip != i) {                                                         \
          T tmp = a[i - 1];                                                    \
          a[i - 1] = a[ip - 1];                                                \
          a[ip - 1] = tmp;                                                     \
        }                                                                      \
      }                                                                        \
    }                                                                          \
  }                                                                            \
  /* Unblocked Crout LU of an m x n panel whose rows are global rows           \
   * off..off+m-1; pivots are stored 1-based relative to the panel top plus    \
   * `off`.  Restates lapack/getf2/getf2_k.c:46-125 step by step: apply the    \
   * earlier swaps to column j, forward-substitute the U part, GEMV update,    \
   * IAMAX (first maximum), swap rows j/jp over columns 0..j, scale by the     \
   * reciprocal only when |pivot| >= TMIN, info = first exact-zero pivot. */   \
  static int PFX##getf2(int m, int n, T *a, int lda, int *ipiv, int off) {     \
    int info = 0;                                                              \
    for (int j = 0; j < n; ++j) {                                              \
      T *b = a + (size_t)j * lda;                                              \
      int len = j < m ? j : m;                                                 \
      for (int i = 0; i < len; ++i) {                                          \
        int ip = ipiv[i + off] - 1 - off;                                      \
        if (ip != i) {                                                         \
          T t = b[i];                                                          \
          b[i] = b[ip];                                                        \
          b[ip] = t;                                                           \
        }                                                                      \
      }                                                                        \
      for (int i = 1; i < len; ++i) {                                          \
        T s = (T)0;                                                            \
        for (int p = 0; p < i; ++p) s += a[(size_t)p * lda + i] * b[p];        \
        b[i] -= s;                                                             \
      }                                                                        \
      if (j < m) {                                                             \
        for (int p = 0; p < j; ++p) {                                          \
          T t = b[p];                                                          \
          if (t == (T)0) continue;                                             \
          const T *ap = a + (size_t)p * lda;                                   \
          for (int i = j; i < m; ++i) b[i] -= ap[i] * t;                       \
        }                                                                      \
        int jp = j;                                                            \
        T best = (T)fabs((double)b[j]);                                        \
        for (int i = j + 1; i < m; ++i) {                                      \
          T v = (T)fabs((double)b[i]);                                         \
          if (v > best) {                                                      \
            best = v;                                                          \
            jp = i;                                                            \
          }                                                                    \
        }                                                                      \
        ipiv[j + off] = jp + 1 + off;                                          \
        T piv = b[jp];                                                         \
        if (piv != (T)0) {                                                     \
          if ((T)fabs((double)piv) >= TMIN) {                                  \
            T r = (T)1 / piv;                                                  \
            if (jp != j) {                                                     \
              for (int c = 0; c <= j; ++c) {                                   \
                T t = a[(size_t)c * lda + j];                                  \
                a[(size_t)c * lda + j] = a[(size_t)c * lda + jp];              \
                a[(size_t)c * lda + jp] = t;                                   \
              }                                                                \
            }                                                                  \
            for (int i = j + 1; i < m; ++i) b[i] *= r;                         \
          }                                                                    \
        } else if (!info) {                                                    \
          info = j + 1;                                                        \
        }                                                                      \
      }                                                                        \
    }                                                                          \
    return info;                                                               \
  }                                                                            \
  /* Right-looking blocked LU (lapack/getrf/getrf_single.c:47-180): factor a   \
   * panel, swap the trailing columns, TRSM with the unit-lower diagonal       \
   * block, GEMM update of the trailing matrix, and finally apply the later    \
   * pivots to the columns left of each panel. */                              \
  int PFX##getrf(int m, int n, T *A, int lda, int *ipiv) {                     \
    if (m <= 0 || n <= 0) return 0;                                            \
    int mn = m < n ? m : n;                                                    \
    const int nb = 64;                                                         \
    int info = 0;                                                              \
    for (int j = 0; j < mn; j += nb) {                                         \
      int jb = mn - j < nb ? mn - j : nb;                                      \
      /* panel rows j..m-1, columns j..j+jb-1; pivots relative to row j */     \
      int *pv = ipiv + j;                                                      \
      int iinfo = PFX##getf2(m - j, jb, A + (size_t)j * lda + j, lda, pv, 0);  \
      if (iinfo && !info) info = iinfo + j;                                    \
      for (int t = 0; t < jb; ++t) pv[t] += j;                                 \
      if (j + jb < n) {                                                        \
        PFX##laswp(n - j - jb, A + (size_t)(j + jb) * lda, lda, j + 1, j + jb, \
                   ipiv, 1);                                                   \
        TRSM('L', 'L', 'N', 'U', jb, n - j - jb, (T)1,                         \
             A + (size_t)j * lda + j, lda, A + (size_t)(j + jb) * lda + j,     \
             lda);                                                             \
        if (j + jb < m)                                                        \
          GEMM('N', 'N', m - j - jb, n - j - jb, jb, (T)-1,                    \
               A + (size_t)j * lda + j + jb, lda,                              \
               A + (size_t)(j + jb) * lda + j, lda, (T)1,                      \
               A + (size_t)(j + jb) * lda + j + jb, lda);                      \
      }                                                                        \
      if (j > 0) PFX##laswp(j, A, lda, j + 1, j + jb, ipiv, 1);                \
    }                                                                          \
    return info;                                                               \
  }                                                                            \
  int PFX##getrs(char trans, int n, int nrhs, const T *A, int lda,            \
                 const int *ipiv, T *B, int ldb) {                             \
    if (n <= 0 || nrhs <= 0) return 0;                                         \
    if (!is_trans(trans)) {                                                    \
      PFX##laswp(nrhs, B, ldb, 1, n, ipiv, 1);                                 \
      TRSM('L', 'L', 'N', 'U', n, nrhs, (T)1, A, lda, B, ldb);                 \
      TRSM('L', 'U', 'N', 'N', n, nrhs, (T)1, A, lda, B, ldb);                 \
    } else {                                                                   \
      TRSM('L', 'U', 'T', 'N', n, nrhs, (T)1, A, lda, B, ldb);                 \
      TRSM('L', 'L', 'T', 'U', n, nrhs, (T)1, A, lda, B, ldb);                 \
      PFX##laswp(nrhs, B, ldb, 1, n, ipiv, -1);                                \
    }                                                                          \
    return 0;                                                                  \
  }

DEFINE_LU(orc_d, double, DBL_MIN, orc_dgemm, orc_dtrsm)
DEFINE_LU(orc_s, float, FLT_MIN, orc_sgemm, orc_strsm)

int orc_dgesv(int n, int nrhs, double *A, int lda, int *ipiv, double *B,
              int ldb) {
  if (n <= 0 || nrhs <= 0) return 0;
  int info = orc_dgetrf(n, n, A, lda, ipiv);
  if (info == 0) orc_dgetrs('N', n, nrhs, A, lda, ipiv, B, ldb);
  return info;
}

/* ------------------------------------------------------------------------ */
/* POTRF                                                                     */
/* ------------------------------------------------------------------------ */
/* potf2_L.c:50-97 / potf2_U.c:50-94 on an nb x nb diagonal block, then the
 * panel TRSM and the SYRK trailing update of potrf_{L,U}_single.c. */
#define DEFINE_POTRF(PFX, T, SQRT)                                             \
  static int PFX##potf2(int lower, int n, T *a, int lda) {                     \
    for (int j = 0; j < n; ++j) {                                              \
      T s = (T)0;                                                              \
      for (int p = 0; p < j; ++p) {                                            \
        T v = lower ? a[(size_t)p * lda + j] : a[(size_t)j * lda + p];         \
        s += v * v;                                                            \
      }                                                                        \
      T ajj = a[(size_t)j * lda + j] - s;                                      \
      if (ajj <= (T)0) {                                                       \
        a[(size_t)j * lda + j] = ajj;                                          \
        return j + 1;                                                          \
      }                                                                        \
      ajj = SQRT(ajj);                                                         \
      a[(size_t)j * lda + j] = ajj;                                            \
      T r = (T)1 / ajj;                                                        \
      for (int i = j + 1; i < n; ++i) {                                        \
        T t = (T)0;                                                            \
        for (int p = 0; p < j; ++p)                                            \
          t += lower ? a[(size_t)p * lda + i] * a[(size_t)p * lda + j]         \
                     : a[(size_t)i * lda + p] * a[(size_t)j * lda + p];        \
        if (lower)                                                             \
          a[(size_t)j * lda + i] = (a[(size_t)j * lda + i] - t) * r;           \
        else                                                                   \
          a[(size_t)i * lda + j] = (a[(size_t)i * lda + j] - t) * r;           \
      }                                                                        \
    }                                                                          \
    return 0;                                                                  \
  }

DEFINE_POTRF(orc_d, double, sqrt)
DEFINE_POTRF(orc_s, float, sqrtf)

int orc_dpotrf(char uplo, int n, double *A, int lda) {
  if (n <= 0) return 0;
  int lower = upc(uplo) == 'L';
  const int nb = 64;
  for (int j = 0; j < n; j += nb) {
    int jb = n - j < nb ? n - j : nb;
    double *d = A + (size_t)j * lda + j;
    int info = orc_dpotf2(lower, jb, d, lda);
    if (info) return info + j;
    int rest = n - j - jb;
    if (rest <= 0) continue;
    if (lower) {
      double *p = A + (size_t)j * lda + j + jb; /* rest x jb */
      orc_dtrsm('R', 'L', 'T', 'N', rest, jb, 1.0, d, lda, p, lda);
      orc_dsyrk('L', 'N', rest, jb, -1.0, p, lda, 1.0,
                A + (size_t)(j + jb) * lda + j + jb, lda);
    } else {
      double *p = A + (size_t)(j + jb) * lda + j; /* jb x rest */
      orc_dtrsm('L', 'U', 'T', 'N', jb, rest, 1.0, d, lda, p, lda);
      orc_dsyrk('U', 'T', rest, jb, -1.0, p, lda, 1.0,
                A + (size_t)(j + jb) * lda + j + jb, lda);
    }
  }
  return 0;
}

int orc_spotrf(char uplo, int n, float *A, int lda) {
  /* single precision, unblocked (test-sized problems only) */
  if (n <= 0) return 0;
  return orc_spotf2(upc(uplo) == 'L', n, A, lda);
}

/* ------------------------------------------------------------------------ */
/* DSGESV                                                                    */
/* ------------------------------------------------------------------------ */
double orc_dlange_inf(int m, int n, const double *A, int lda) {
  double best = 0.0;
  for (int i = 0; i < m; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) s += fabs(A[(size_t)j * lda + i]);
    if (s > best || isnan(s)) best = s;
  }
  return best;
}

static int lag2s(int m, int n, const double *A, int lda, float *S, int lds) {
  /* dlag2s.f:136-145: abort with info=1 if any |a| > SLAMCH('O') */
  const double rmax = (double)FLT_MAX;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double v = A[(size_t)j * lda + i];
      if (v < -rmax || v > rmax) return 1;
      S[(size_t)j * lds + i] = (float)v;
    }
  return 0;
}

static int idamax0(int n, const double *x) {
  int best = 0;
  double bv = fabs(x[0]);
  for (int i = 1; i < n; ++i)
    if (fabs(x[i]) > bv) {
      bv = fabs(x[i]);
      best = i;
    }
  return best;
}

int orc_dsgesv(int n, int nrhs, double *A, int lda, int *ipiv, const double *B,
               int ldb, double *X, int ldx, int *iter) {
  *iter = 0;
  if (n <= 0) return 0;
  const int itermax = 30;
  double anrm = orc_dlange_inf(n, n, A, lda);
  double eps = DBL_EPSILON * 0.5; /* DLAMCH('Epsilon') */
  double cte = anrm * eps * sqrt((double)n) * 1.0;
  float *sa = (float *)malloc(sizeof(float) * (size_t)n * n);
  float *sx = (float *)malloc(sizeof(float) * (size_t)n * nrhs);
  double *w = (double *)malloc(sizeof(double) * (size_t)n * nrhs);
  int info = 0;
  if (lag2s(n, nrhs, B, ldb, sx, n)) {
    *iter = -2;
    goto fallback;
  }
  if (lag2s(n, n, A, lda, sa, n)) {
    *iter = -2;
    goto fallback;
  }
  if (orc_sgetrf(n, n, sa, n, ipiv)) {
    *iter = -3;
    goto fallback;
  }
  orc_sgetrs('N', n, nrhs, sa, n, ipiv, sx, n);
  for (int j = 0; j < nrhs; ++j)
    for (int i = 0; i < n; ++i)
      X[(size_t)j * ldx + i] = (double)sx[(size_t)j * n + i];
  for (int it = 0; it <= itermax; ++it) {
    for (int j = 0; j < nrhs; ++j)
      memcpy(w + (size_t)j * n, B + (size_t)j * ldb, sizeof(double) * n);
    orc_dgemm('N', 'N', n, nrhs, n, -1.0, A, lda, X, ldx, 1.0, w, n);
    int ok = 1;
    for (int j = 0; j < nrhs; ++j) {
      double xn = fabs(X[(size_t)j * ldx + idamax0(n, X + (size_t)j * ldx)]);
      double rn = fabs(w[(size_t)j * n + idamax0(n, w + (size_t)j * n)]);
      if (rn > xn * cte) {
        ok = 0;
        break;
      }
    }
    if (ok) {
      *iter = it;
      free(sa);
      free(sx);
      free(w);
      return 0;
    }
    if (it == itermax) break;
    if (lag2s(n, nrhs, w, n, sx, n)) {
      *iter = -2;
      goto fallback;
    }
    orc_sgetrs('N', n, nrhs, sa, n, ipiv, sx, n);
    for (int j = 0; j < nrhs; ++j)
      for (int i = 0; i < n; ++i)
        X[(size_t)j * ldx + i] += (double)sx[(size_t)j * n + i];
  }
  *iter = -itermax - 1;
fallback:
  free(sa);
  free(sx);
  free(w);
  info = orc_dgetrf(n, n, A, lda, ipiv);
  if (info) return info;
  for (int j = 0; j < nrhs; ++j)
    memcpy(X + (size_t)j * ldx, B + (size_t)j * ldb, sizeof(double) * n);
  orc_dgetrs('N', n, nrhs, A, lda, ipiv, X, ldx);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* TRMM / SYR2K / GEMMT                                                      */
/* ------------------------------------------------------------------------ */
/* driver/level3/trmm_L.c, trmm_R.c (interface/trsm.c built as TRMM):
 * B = alpha*op(T)*B (side L) or alpha*B*op(T) (side R), T the uplo triangle of
 * A with a unit diagonal for diag 'U'; alpha == 0 zeroes B (GEMM_BETA). */
void orc_dtrmm(char side, char uplo, char transa, char diag, int m, int n, double alpha,
               const double *A, int lda, double *B, int ldb) {
  if (m <= 0 || n <= 0) return;
  const int left = upc(side) == 'L', lower = upc(uplo) == 'L';
  const int tr = upc(transa) == 'T' || upc(transa) == 'C', unit = upc(diag) == 'U';
  if (alpha == 0.0) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) B[(size_t)j * ldb + i] = 0.0;
    return;
  }
  const int na = left ? m : n;
  double *T = (double *)calloc((size_t)na * na, sizeof(double));
  for (int j = 0; j < na; ++j)
    for (int i = 0; i < na; ++i) {
      double v = 0.0;
      if (i == j) v = unit ? 1.0 : A[(size_t)j * lda + i];
      else if (lower ? i > j : i < j) v = A[(size_t)j * lda + i];
      T[(size_t)j * na + i] = v;
    }
  double *W = (double *)malloc(sizeof(double) * (size_t)m * n);
  for (int j = 0; j < n; ++j) memcpy(W + (size_t)j * m, B + (size_t)j * ldb, sizeof(double) * m);
  if (left)
    orc_dgemm(tr ? 'T' : 'N', 'N', m, n, m, alpha, T, na, W, m, 0.0, B, ldb);
  else
    orc_dgemm('N', tr ? 'T' : 'N', m, n, n, alpha, W, m, T, na, 0.0, B, ldb);
  free(T);
  free(W);
}

/* driver/level3/level3_syr2k.c: C = alpha*op(A)*op(B)^T + alpha*op(B)*op(A)^T
 * + beta*C on the uplo triangle (trans 'N': A, B n x k; 'T': k x n). */
void orc_dsyr2k(char uplo, char trans, int n, int k, double alpha, const double *A, int lda,
                const double *B, int ldb, double beta, double *C, int ldc) {
  if (n <= 0) return;
  const int lower = upc(uplo) == 'L', tr = upc(trans) != 'N';
  for (int j = 0; j < n; ++j)
    for (int i = lower ? j : 0; i < (lower ? n : j + 1); ++i) {
      double s = 0.0;
      if (alpha != 0.0)
        for (int p = 0; p < k; ++p) {
          const double aip = tr ? A[(size_t)i * lda + p] : A[(size_t)p * lda + i];
          const double bjp = tr ? B[(size_t)j * ldb + p] : B[(size_t)p * ldb + j];
          const double bip = tr ? B[(size_t)i * ldb + p] : B[(size_t)p * ldb + i];
          const double ajp = tr ? A[(size_t)j * lda + p] : A[(size_t)p * lda + j];
          s += aip * bjp + bip * ajp;
        }
      double *c = C + (size_t)j * ldc + i;
      *c = (beta == 0.0 ? 0.0 : beta * *c) + alpha * s;
    }
}

/* interface/gemmt.c: C = alpha*op(A)*op(B) + beta*C on the uplo triangle of
 * the m x m matrix C. */
void orc_dgemmt(char uplo, char transa, char transb, int m, int k, double alpha,
                const double *A, int lda, const double *B, int ldb, double beta, double *C,
                int ldc) {
  if (m <= 0) return;
  const int lower = upc(uplo) == 'L';
  const int ta = upc(transa) == 'T' || upc(transa) == 'C';
  const int tb = upc(transb) == 'T' || upc(transb) == 'C';
  for (int j = 0; j < m; ++j)
    for (int i = lower ? j : 0; i < (lower ? m : j + 1); ++i) {
      double s = 0.0;
      if (alpha != 0.0)
        for (int p = 0; p < k; ++p) {
          const double a = ta ? A[(size_t)i * lda + p] : A[(size_t)p * lda + i];
          const double b = tb ? B[(size_t)p * ldb + j] : B[(size_t)j * ldb + p];
          s += a * b;
        }
      double *c = C + (size_t)j * ldc + i;
      *c = (beta == 0.0 ? 0.0 : beta * *c) + alpha * s;
    }
}

/* ------------------------------------------------------------------------ */
/* DPOTRS / DSPOSV                                                           */
/* ------------------------------------------------------------------------ */
/* lapack-netlib/SRC/dpotrs.f:135-160: two triangular solves with the factor. */
int orc_dpotrs(char uplo, int n, int nrhs, const double *A, int lda, double *B, int ldb) {
  if (n <= 0 || nrhs <= 0) return 0;
  if (upc(uplo) == 'L') {
    orc_dtrsm('L', 'L', 'N', 'N', n, nrhs, 1.0, A, lda, B, ldb);
    orc_dtrsm('L', 'L', 'T', 'N', n, nrhs, 1.0, A, lda, B, ldb);
  } else {
    orc_dtrsm('L', 'U', 'T', 'N', n, nrhs, 1.0, A, lda, B, ldb);
    orc_dtrsm('L', 'U', 'N', 'N', n, nrhs, 1.0, A, lda, B, ldb);
  }
  return 0;
}

static void spotrs(int lower, int n, int nrhs, const float *A, int lda, float *B, int ldb) {
  if (lower) {
    orc_strsm('L', 'L', 'N', 'N', n, nrhs, 1.0f, A, lda, B, ldb);
    orc_strsm('L', 'L', 'T', 'N', n, nrhs, 1.0f, A, lda, B, ldb);
  } else {
    orc_strsm('L', 'U', 'T', 'N', n, nrhs, 1.0f, A, lda, B, ldb);
    orc_strsm('L', 'U', 'N', 'N', n, nrhs, 1.0f, A, lda, B, ldb);
  }
}

/* element (i, j) of a symmetric matrix held in one triangle */
static double sym_at(int lower, const double *A, int lda, int i, int j) {
  if (lower ? i >= j : i <= j) return A[(size_t)j * lda + i];
  return A[(size_t)i * lda + j];
}

/* DLANSY('I') (dlansy.f: infinity norm from the stored triangle) */
static double dlansy_inf(int lower, int n, const double *A, int lda) {
  double best = 0.0;
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) s += fabs(sym_at(lower, A, lda, i, j));
    if (s > best || isnan(s)) best = s;
  }
  return best;
}

/* W = W - A X with the stored triangle (DSYMM('L', uplo, ..., -1, A, X, 1, W)) */
static void dsymm_minus(int lower, int n, int nrhs, const double *A, int lda, const double *X,
                        int ldx, double *W, int ldw) {
  for (int c = 0; c < nrhs; ++c)
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int j = 0; j < n; ++j) s += sym_at(lower, A, lda, i, j) * X[(size_t)c * ldx + j];
      W[(size_t)c * ldw + i] -= s;
    }
}

/* DLAT2S (dlat2s.f): FP32 copy of the stored triangle; 1 on overflow */
static int lat2s(int lower, int n, const double *A, int lda, float *S, int lds) {
  const double rmax = (double)FLT_MAX;
  for (int j = 0; j < n; ++j)
    for (int i = lower ? j : 0; i < (lower ? n : j + 1); ++i) {
      const double v = A[(size_t)j * lda + i];
      if (v < -rmax || v > rmax) return 1;
      S[(size_t)j * lds + i] = (float)v;
    }
  return 0;
}

/* lapack-netlib/SRC/dsposv.f:232-434 */
int orc_dsposv(char uplo, int n, int nrhs, double *A, int lda, const double *B, int ldb,
               double *X, int ldx, int *iter) {
  *iter = 0;
  if (n <= 0) return 0;
  const int lower = upc(uplo) == 'L';
  const int itermax = 30;
  const double anrm = dlansy_inf(lower, n, A, lda);
  const double eps = DBL_EPSILON * 0.5; /* DLAMCH('Epsilon') */
  const double cte = anrm * eps * sqrt((double)n) * 1.0;
  float *sa = (float *)calloc((size_t)n * n, sizeof(float));
  float *sx = (float *)malloc(sizeof(float) * (size_t)n * nrhs);
  double *w = (double *)malloc(sizeof(double) * (size_t)n * nrhs);
  int info = 0;
  if (lag2s(n, nrhs, B, ldb, sx, n)) {
    *iter = -2;
    goto fallback;
  }
  if (lat2s(lower, n, A, lda, sa, n)) {
    *iter = -2;
    goto fallback;
  }
  if (orc_spotf2(lower, n, sa, n)) {
    *iter = -3;
    goto fallback;
  }
  spotrs(lower, n, nrhs, sa, n, sx, n);
  for (int j = 0; j < nrhs; ++j)
    for (int i = 0; i < n; ++i) X[(size_t)j * ldx + i] = (double)sx[(size_t)j * n + i];
  for (int it = 0; it <= itermax; ++it) {
    for (int j = 0; j < nrhs; ++j) memcpy(w + (size_t)j * n, B + (size_t)j * ldb, sizeof(double) * n);
    dsymm_minus(lower, n, nrhs, A, lda, X, ldx, w, n);
    int ok = 1;
    for (int j = 0; j < nrhs; ++j) {
      double xn = fabs(X[(size_t)j * ldx + idamax0(n, X + (size_t)j * ldx)]);
      double rn = fabs(w[(size_t)j * n + idamax0(n, w + (size_t)j * n)]);
      if (rn > xn * cte) {
        ok = 0;
        break;
      }
    }
    if (ok) {
      *iter = it;
      free(sa);
      free(sx);
      free(w);
      return 0;
    }
    if (it == itermax) break;
    if (lag2s(n, nrhs, w, n, sx, n)) {
      *iter = -2;
      goto fallback;
    }
    spotrs(lower, n, nrhs, sa, n, sx, n);
    for (int j = 0; j < nrhs; ++j)
      for (int i = 0; i < n; ++i) X[(size_t)j * ldx + i] += (double)sx[(size_t)j * n + i];
  }
  *iter = -itermax - 1;
fallback:
  free(sa);
  free(sx);
  free(w);
  info = orc_dpotrf(uplo, n, A, lda);
  if (info) return info;
  for (int j = 0; j < nrhs; ++j) memcpy(X + (size_t)j * ldx, B + (size_t)j * ldb, sizeof(double) * n);
  orc_dpotrs(uplo, n, nrhs, A, lda, X, ldx);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Complex GEMM: ZGEMM/CGEMM and the 3M forms ZGEMM3M/CGEMM3M               */
/* ------------------------------------------------------------------------ */
/* op codes of interface/gemm.c:253-268 compiled with COMPLEX: N 0, T 1,
 * R 2 (conjugate, no transpose), C 3 (conjugate transpose); -1 invalid. */
static int ztrans(char t) {
  if (t >= 'a' && t <= 'z') t = (char)(t - 32);
  return t == 'N' ? 0 : t == 'T' ? 1 : t == 'R' ? 2 : t == 'C' ? 3 : -1;
}

/* C <- beta C, kernel/generic/zgemm_beta.c:38-100: beta = 0 stores zeros;
 * level3.c:229-249 skips beta = (1, 0). */
#define DEFINE_ZBETA(NAME, T)                                                  \
  static void NAME(int m, int n, T br, T bi, T *C, int ldc) {                  \
    if (br == (T)1 && bi == (T)0) return;                                      \
    for (int j = 0; j < n; ++j)                                                \
      for (int i = 0; i < m; ++i) {                                            \
        T *c = C + 2 * ((size_t)j * ldc + i);                                  \
        if (br == (T)0 && bi == (T)0) {                                        \
          c[0] = (T)0;                                                         \
          c[1] = (T)0;                                                         \
        } else {                                                               \
          T r = br * c[0] - bi * c[1], s = br * c[1] + bi * c[0];              \
          c[0] = r;                                                            \
          c[1] = s;                                                            \
        }                                                                      \
      }                                                                        \
  }
DEFINE_ZBETA(zbeta_d, double)
DEFINE_ZBETA(zbeta_s, float)

/* op(X)(i, p) of a complex matrix stored column-major with leading dimension
 * ld: transposed for codes 1 and 3, conjugated for codes 2 and 3. */
#define ZELEM(T, X, ld, code, i, p, re, im)                                    \
  do {                                                                         \
    const T *e_ = ((code) & 1) ? (X) + 2 * ((size_t)(i) * (ld) + (p))          \
                               : (X) + 2 * ((size_t)(p) * (ld) + (i));         \
    re = e_[0];                                                                \
    im = (code) >= 2 ? -e_[1] : e_[1];                                         \
  } while (0)

/* ZGEMM / CGEMM: level3.c:229-259 (beta, then nothing when k = 0 or
 * alpha = 0) and the complex kernels' accumulate-then-scale
 * (kernel/generic/zgemmkernel_2x2.c: c += alpha * sum op(a) op(b)). */
#define DEFINE_ZGEMM(NAME, T, BETA)                                            \
  void NAME(char transa, char transb, int m, int n, int k, const T *alpha,     \
            const T *A, int lda, const T *B, int ldb, const T *beta, T *C,     \
            int ldc) {                                                         \
    if (m <= 0 || n <= 0) return;                                              \
    const int ta = ztrans(transa), tb = ztrans(transb);                        \
    const T ar = alpha[0], ai = alpha[1];                                      \
    BETA(m, n, beta[0], beta[1], C, ldc);                                      \
    if (k <= 0 || (ar == (T)0 && ai == (T)0)) return;                          \
    int nthr = orc_get_threads();                                              \
    if ((double)m * n * k < 2e5) nthr = 1;                                     \
    _Pragma("omp parallel for num_threads(nthr) schedule(dynamic, 4)")         \
    for (int j = 0; j < n; ++j)                                                \
      for (int i = 0; i < m; ++i) {                                            \
        T sr = (T)0, si = (T)0;                                                \
        for (int p = 0; p < k; ++p) {                                          \
          T a_r, a_i, b_r, b_i;                                                \
          ZELEM(T, A, lda, ta, i, p, a_r, a_i);                                \
          ZELEM(T, B, ldb, tb, p, j, b_r, b_i);                                \
          sr += a_r * b_r - a_i * b_i;                                         \
          si += a_r * b_i + a_i * b_r;                                         \
        }                                                                      \
        T *c = C + 2 * ((size_t)j * ldc + i);                                  \
        c[0] += ar * sr - ai * si;                                             \
        c[1] += ar * si + ai * sr;                                             \
      }                                                                        \
  }
DEFINE_ZGEMM(orc_zgemm, double, zbeta_d)
DEFINE_ZGEMM(orc_cgemm, float, zbeta_s)

/* ZGEMM3M / CGEMM3M, driver/level3/gemm3m_level3.c: B' = alpha op(B) formed
 * in the copies of B (zgemm3m_ncopy_*.c REAL_PART / IMAGE_PART), then three
 * real products T1 = (Ar + Ai)(B'r + B'i), T2 = Ar B'r, T3 = Ai B'i added to
 * C with the ALPHA5..ALPHA18 signs of the NN case (gemm3m_level3.c:155-168):
 * Im += T1; Re += T2, Im -= T2; Re -= T3, Im -= T3. */
#define DEFINE_ZGEMM3M(NAME, T, BETA)                                          \
  void NAME(char transa, char transb, int m, int n, int k, const T *alpha,     \
            const T *A, int lda, const T *B, int ldb, const T *beta, T *C,     \
            int ldc) {                                                         \
    if (m <= 0 || n <= 0) return;                                              \
    const int ta = ztrans(transa), tb = ztrans(transb);                        \
    const T ar = alpha[0], ai = alpha[1];                                      \
    BETA(m, n, beta[0], beta[1], C, ldc);                                      \
    if (k <= 0 || (ar == (T)0 && ai == (T)0)) return;                          \
    T *bp = (T *)malloc(sizeof(T) * 3 * (size_t)k * n); /* B'r, B'i, sum */    \
    for (int j = 0; j < n; ++j)                                                \
      for (int p = 0; p < k; ++p) {                                            \
        T b_r, b_i;                                                            \
        ZELEM(T, B, ldb, tb, p, j, b_r, b_i);                                  \
        const T wr = ar * b_r - ai * b_i, wi = ai * b_r + ar * b_i;            \
        const size_t e = (size_t)j * k + p, kn = (size_t)k * n;                \
        bp[e] = wr;                                                            \
        bp[kn + e] = wi;                                                       \
        bp[2 * kn + e] = wr + wi;                                              \
      }                                                                        \
    int nthr = orc_get_threads();                                              \
    if ((double)m * n * k < 2e5) nthr = 1;                                     \
    _Pragma("omp parallel for num_threads(nthr) schedule(dynamic, 4)")         \
    for (int j = 0; j < n; ++j)                                                \
      for (int i = 0; i < m; ++i) {                                            \
        T t1 = (T)0, t2 = (T)0, t3 = (T)0;                                     \
        const size_t kn = (size_t)k * n;                                       \
        for (int p = 0; p < k; ++p) {                                          \
          T a_r, a_i;                                                          \
          ZELEM(T, A, lda, ta, i, p, a_r, a_i);                                \
          const size_t e = (size_t)j * k + p;                                  \
          t1 += (a_r + a_i) * bp[2 * kn + e];                                  \
          t2 += a_r * bp[e];                                                   \
          t3 += a_i * bp[kn + e];                                              \
        }                                                                      \
        T *c = C + 2 * ((size_t)j * ldc + i);                                  \
        c[1] += t1;                                                            \
        c[0] += t2;                                                            \
        c[1] -= t2;                                                            \
        c[0] -= t3;                                                            \
        c[1] -= t3;                                                            \
      }                                                                        \
    free(bp);                                                                  \
  }
DEFINE_ZGEMM3M(orc_zgemm3m, double, zbeta_d)
DEFINE_ZGEMM3M(orc_cgemm3m, float, zbeta_s)

/* ------------------------------------------------------------------------ */
/* Grouped batch on the host cores                                           */
/* ------------------------------------------------------------------------ */
/* One problem per thread (the inner routines run single-threaded inside the
 * parallel loop: nested OpenMP regions are not activated), dynamic schedule
 * over the problems as gemm_batch_thread.c:79-156 hands them to its threads. */
void orc_batch(const orc_batch_problem *probs, int count) {
  int nthr = orc_get_threads();
#pragma omp parallel for num_threads(nthr) schedule(dynamic, 1)
  for (int i = 0; i < count; ++i) {
    const orc_batch_problem *p = &probs[i];
    if (p->type == 0) {
      orc_dgemm(p->transa, p->transb, p->m, p->n, p->k, p->alpha, (const double *)p->A, p->lda,
                (const double *)p->B, p->ldb, p->beta, (double *)p->C, p->ldc);
    } else if (p->type == 1) {
      int info = orc_dgesv(p->n, p->k, (double *)p->A, p->lda, (int *)p->C, (double *)p->B,
                           p->ldb);
      if (p->info) *p->info = info;
    } else if (p->type == 2) {
      int info = orc_dpotrf(p->uplo, p->n, (double *)p->A, p->lda);
      if (p->info) *p->info = info;
    }
  }
}
