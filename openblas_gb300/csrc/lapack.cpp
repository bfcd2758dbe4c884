// LAPACK entry points of libgbblas: dgetrf_, dgetrs_, dgesv_, dpotrf_,
// dlaswp_ and their device-pointer variants.
//
// Argument checks, xerbla positions, `*Info = -info` on argument errors and
// the quick returns restate interface/lapack/getrf.c:53-133, getrs.c:63-152,
// gesv.c:63-161, potrf.c:63-150 and laswp.c:55-110.  The factorisations run
// on the GPU (lapack_kernels.cu); host-pointer calls stage A/B through the
// library stream and copy the results (and ipiv) back before returning.
#include <string.h>

#include "gb_internal.h"
#include "lapack_internal.h"
#include "operand.h"

using namespace gb;

namespace {

// Device copy of a host int vector (ipiv) of `n` entries; used in place when
// the caller's pointer is already device memory.
struct IntVec {
  int *user;
  int64_t n;
  int *dev = nullptr;
  bool staged = false;
  Scratch buf;
  IntVec(int *p, int64_t cnt) : user(p), n(cnt) {}
  int bind(bool copy_in, cudaStream_t s) {
    if (n <= 0) return GB_SUCCESS;
    if (is_device_pointer(user)) {
      dev = user;
      return GB_SUCCESS;
    }
    new (&buf) Scratch((size_t)n * sizeof(int), s);
    if (!buf.p) return GB_ERR_ALLOC;
    dev = buf.as<int>();
    staged = true;
    if (copy_in) GB_CUDA(cudaMemcpyAsync(dev, user, n * sizeof(int), cudaMemcpyHostToDevice, s));
    return GB_SUCCESS;
  }
  int unbind(cudaStream_t s) {
    if (!staged) return GB_SUCCESS;
    GB_CUDA(cudaMemcpyAsync(user, dev, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    return GB_SUCCESS;
  }
};

// One int of device scratch for `info`, read back after the stream syncs.
struct DevInfo {
  Scratch buf;
  explicit DevInfo(cudaStream_t s) : buf(sizeof(int) * 4, s) {}
  int *d() const { return buf.as<int>(); }
  int read(cudaStream_t s, int *out) {
    int h = 0;
    GB_CUDA(cudaMemcpyAsync(&h, d(), sizeof(int), cudaMemcpyDeviceToHost, s));
    int st = finish_blocking(s);
    if (st) return st;
    *out = h;
    return GB_SUCCESS;
  }
};

int getrf_blocking(int64_t m, int64_t n, double *A, int64_t lda, int *ipiv, int *info) {
  int st = ensure_init();
  if (st) return st;
  cudaStream_t s = stream();
  Operand a(A, m, n, lda, 8);
  IntVec p(ipiv, m < n ? m : n);
  if ((st = a.bind(true, s)) || (st = p.bind(false, s))) return st;
  DevInfo di(s);
  if (!di.buf.p) return GB_ERR_ALLOC;
  const int mode = gb_get_dgemm_mode() == GB_DGEMM_NATIVE ? 0 : 1;
  if ((st = getrf_device_mode<double>(m, n, a.d<double>(), a.dld, p.dev, di.d(), mode, s)))
    return st;
  if ((st = a.unbind(s)) || (st = p.unbind(s))) return st;
  return di.read(s, info);
}

}  // namespace

extern "C" {

int dgetrf_(const blasint *M, const blasint *N, double *a, const blasint *ldA, blasint *ipiv,
            blasint *Info) {
  int64_t m = *M, n = *N, lda = *ldA;
  int info = 0;
  if (lda < (m > 1 ? m : 1)) info = 4;
  if (n < 0) info = 2;
  if (m < 0) info = 1;
  if (info) {
    call_xerbla("DGETRF", info);
    *Info = -info;
    return 0;
  }
  *Info = 0;
  if (m == 0 || n == 0) return 0;
  int out = 0;
  if (getrf_blocking(m, n, a, lda, ipiv, &out) == GB_SUCCESS) *Info = out;
  return 0;
}

int dgetrs_(const char *TRANS, const blasint *N, const blasint *NRHS, const double *a,
            const blasint *ldA, const blasint *ipiv, double *b, const blasint *ldB,
            blasint *Info) {
  char t = upch(TRANS);
  int trans = (t == 'N' || t == 'R') ? 0 : (t == 'T' || t == 'C') ? 1 : -1;
  int64_t n = *N, nrhs = *NRHS, lda = *ldA, ldb = *ldB;
  int info = 0;
  if (ldb < (n > 1 ? n : 1)) info = 8;
  if (lda < (n > 1 ? n : 1)) info = 5;
  if (nrhs < 0) info = 3;
  if (n < 0) info = 2;
  if (trans < 0) info = 1;
  if (info) {
    // interface/lapack/getrs.c:124-127 reports through xerbla only
    call_xerbla("DGETRS", info);
    return 0;
  }
  *Info = 0;
  if (n == 0 || nrhs == 0) return 0;
  if (ensure_init()) return 0;
  cudaStream_t s = stream();
  Operand A(a, n, n, lda, 8), B(b, n, nrhs, ldb, 8);
  IntVec p(const_cast<int *>(ipiv), n);
  if (A.bind(true, s) || B.bind(true, s) || p.bind(true, s)) return 0;
  if (getrs_device<double>(trans, n, nrhs, A.d<double>(), A.dld, p.dev, B.d<double>(), B.dld, s))
    return 0;
  B.unbind(s);
  finish_blocking(s);
  return 0;
}

int dgesv_(const blasint *N, const blasint *NRHS, double *a, const blasint *ldA, blasint *ipiv,
           double *b, const blasint *ldB, blasint *Info) {
  int64_t n = *N, nrhs = *NRHS, lda = *ldA, ldb = *ldB;
  int info = 0;
  if (ldb < (n > 1 ? n : 1)) info = 7;
  if (lda < (n > 1 ? n : 1)) info = 4;
  if (nrhs < 0) info = 2;
  if (n < 0) info = 1;
  if (info) {
    call_xerbla("DGESV", info);
    *Info = -info;
    return 0;
  }
  *Info = 0;
  if (n == 0 || nrhs == 0) return 0;
  if (ensure_init()) return 0;
  cudaStream_t s = stream();
  Operand A(a, n, n, lda, 8), B(b, n, nrhs, ldb, 8);
  IntVec p(ipiv, n);
  if (A.bind(true, s) || B.bind(true, s) || p.bind(false, s)) return 0;
  DevInfo di(s);
  if (!di.buf.p) return 0;
  const int mode = gb_get_dgemm_mode() == GB_DGEMM_NATIVE ? 0 : 1;
  if (getrf_device_mode<double>(n, n, A.d<double>(), A.dld, p.dev, di.d(), mode, s)) return 0;
  int h = 0;
  if (di.read(s, &h)) return 0;
  // interface/lapack/gesv.c:131-135: solve only when the factorisation is regular
  if (h == 0 &&
      getrs_device<double>(0, n, nrhs, A.d<double>(), A.dld, p.dev, B.d<double>(), B.dld, s))
    return 0;
  A.unbind(s);
  p.unbind(s);
  if (h == 0) B.unbind(s);
  if (finish_blocking(s)) return 0;
  *Info = h;
  return 0;
}

int dpotrf_(const char *UPLO, const blasint *N, double *a, const blasint *ldA, blasint *Info) {
  char u = upch(UPLO);
  int uplo = u == 'U' ? 0 : u == 'L' ? 1 : -1;
  int64_t n = *N, lda = *ldA;
  int info = 0;
  if (lda < (n > 1 ? n : 1)) info = 4;
  if (n < 0) info = 2;
  if (uplo < 0) info = 1;
  if (info) {
    call_xerbla("DPOTRF", info);
    *Info = -info;
    return 0;
  }
  *Info = 0;
  if (n == 0) return 0;
  if (ensure_init()) return 0;
  cudaStream_t s = stream();
  Operand A(a, n, n, lda, 8);
  if (A.bind(true, s)) return 0;
  DevInfo di(s);
  if (!di.buf.p) return 0;
  const int mode = gb_get_dgemm_mode() == GB_DGEMM_NATIVE ? 0 : 1;
  if (potrf_device(uplo, n, A.d<double>(), A.dld, di.d(), mode, s)) return 0;
  A.unbind(s);
  int h = 0;
  if (di.read(s, &h)) return 0;
  *Info = h;
  return 0;
}

// lapack-netlib/SRC/dpotrs.f:109-160 (the reference builds dpotrs from
// lapack-netlib): argument checks in order UPLO, N, NRHS, LDA, LDB, quick
// return, then the two triangular solves with the Cholesky factor.
int dpotrs_(const char *UPLO, const blasint *N, const blasint *NRHS, const double *a,
            const blasint *ldA, double *b, const blasint *ldB, blasint *Info) {
  char u = upch(UPLO);
  int uplo = u == 'U' ? 0 : u == 'L' ? 1 : -1;
  int64_t n = *N, nrhs = *NRHS, lda = *ldA, ldb = *ldB;
  int info = 0;
  if (uplo < 0) info = 1;
  else if (n < 0) info = 2;
  else if (nrhs < 0) info = 3;
  else if (lda < (n > 1 ? n : 1)) info = 5;
  else if (ldb < (n > 1 ? n : 1)) info = 7;
  if (info) {
    call_xerbla("DPOTRS", info);
    *Info = -info;
    return 0;
  }
  *Info = 0;
  if (n == 0 || nrhs == 0) return 0;
  if (ensure_init()) return 0;
  cudaStream_t s = stream();
  Operand A(a, n, n, lda, 8), B(b, n, nrhs, ldb, 8);
  if (A.bind(true, s) || B.bind(true, s)) return 0;
  if (potrs_device(uplo, n, nrhs, A.d<double>(), A.dld, B.d<double>(), B.dld, s)) return 0;
  B.unbind(s);
  finish_blocking(s);
  return 0;
}

int dlaswp_(const blasint *N, double *a, const blasint *LDA, const blasint *K1, const blasint *K2,
            const blasint *ipiv, const blasint *INCX) {
  int64_t n = *N, lda = *LDA, k1 = *K1, k2 = *K2, incx = *INCX;
  // interface/lapack/laswp.c:75: incx == 0 or n <= 0 is a no-op
  if (incx == 0 || n <= 0) return 0;
  if (k2 < k1) return 0;
  if (ensure_init()) return 0;
  cudaStream_t s = stream();
  // rows touched: 1..max(k2, max pivot); stage the whole leading block
  int64_t rows = k2;
  const int64_t ainc = incx < 0 ? -incx : incx;
  // entries the interchanges read: row i uses ipiv[(k1-1) + (i-k1)*|incx|]
  // (0-based), i = k1..k2, so no more than the caller has to supply
  const int64_t npiv = (k1 - 1) + (k2 - k1) * ainc + 1;
  bool pdev = is_device_pointer(ipiv);
  if (!pdev)
    for (int64_t t = 0; t < npiv; ++t)
      if (ipiv[t] > rows) rows = ipiv[t];
  if (pdev) rows = lda;
  Operand A(a, rows, n, lda, 8);
  IntVec p(const_cast<int *>(ipiv), npiv);
  if (A.bind(true, s) || p.bind(true, s)) return 0;
  if (laswp_device<double>(n, A.d<double>(), A.dld, k1, k2, p.dev, incx, s)) return 0;
  A.unbind(s);
  finish_blocking(s);
  return 0;
}

// ---------------------------------------------------------------------------
// device-pointer variants
// ---------------------------------------------------------------------------
int gb_dgetrf_dev(int64_t m, int64_t n, double *A, int64_t lda, int *ipiv, int *info) {
  int code = 0;
  if (lda < (m > 1 ? m : 1)) code = 4;
  if (n < 0) code = 2;
  if (m < 0) code = 1;
  if (code) {
    call_xerbla("DGETRF", code);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  if (m == 0 || n == 0) {
    GB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), stream()));
    return GB_SUCCESS;
  }
  const int mode = gb_get_dgemm_mode() == GB_DGEMM_NATIVE ? 0 : 1;
  return getrf_device_mode<double>(m, n, A, lda, ipiv, info, mode, stream());
}

int gb_dgetrs_dev(char trans, int64_t n, int64_t nrhs, const double *A, int64_t lda,
                  const int *ipiv, double *B, int64_t ldb) {
  char t = upch(trans);
  int tr = (t == 'N' || t == 'R') ? 0 : (t == 'T' || t == 'C') ? 1 : -1;
  int code = 0;
  if (ldb < (n > 1 ? n : 1)) code = 8;
  if (lda < (n > 1 ? n : 1)) code = 5;
  if (nrhs < 0) code = 3;
  if (n < 0) code = 2;
  if (tr < 0) code = 1;
  if (code) {
    call_xerbla("DGETRS", code);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  return getrs_device<double>(tr, n, nrhs, A, lda, ipiv, B, ldb, stream());
}

int gb_sgetrf_dev(int64_t m, int64_t n, float *A, int64_t lda, int *ipiv, int *info) {
  int code = 0;
  if (lda < (m > 1 ? m : 1)) code = 4;
  if (n < 0) code = 2;
  if (m < 0) code = 1;
  if (code) {
    call_xerbla("SGETRF", code);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  if (m == 0 || n == 0) {
    GB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), stream()));
    return GB_SUCCESS;
  }
  return getrf_device<float>(m, n, A, lda, ipiv, info, stream());
}

int gb_sgetrs_dev(char trans, int64_t n, int64_t nrhs, const float *A, int64_t lda,
                  const int *ipiv, float *B, int64_t ldb) {
  char t = upch(trans);
  int tr = (t == 'N' || t == 'R') ? 0 : (t == 'T' || t == 'C') ? 1 : -1;
  int code = 0;
  if (ldb < (n > 1 ? n : 1)) code = 8;
  if (lda < (n > 1 ? n : 1)) code = 5;
  if (nrhs < 0) code = 3;
  if (n < 0) code = 2;
  if (tr < 0) code = 1;
  if (code) {
    call_xerbla("SGETRS", code);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  return getrs_device<float>(tr, n, nrhs, A, lda, ipiv, B, ldb, stream());
}

int gb_dlaswp_dev(int64_t n, double *A, int64_t lda, int64_t k1, int64_t k2, const int *ipiv,
                  int64_t incx) {
  int st = ensure_init();
  if (st) return st;
  return laswp_device<double>(n, A, lda, k1, k2, ipiv, incx, stream());
}

int gb_dpotrf_dev(char uplo, int64_t n, double *A, int64_t lda, int *info) {
  char u = upch(uplo);
  int up = u == 'U' ? 0 : u == 'L' ? 1 : -1;
  int code = 0;
  if (lda < (n > 1 ? n : 1)) code = 4;
  if (n < 0) code = 2;
  if (up < 0) code = 1;
  if (code) {
    call_xerbla("DPOTRF", code);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  if (n == 0) {
    GB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), stream()));
    return GB_SUCCESS;
  }
  const int mode = gb_get_dgemm_mode() == GB_DGEMM_NATIVE ? 0 : 1;
  return potrf_device(up, n, A, lda, info, mode, stream());
}

int gb_dpotrs_dev(char uplo, int64_t n, int64_t nrhs, const double *A, int64_t lda, double *B,
                  int64_t ldb) {
  const char u = upch(uplo);
  const int up = u == 'U' ? 0 : u == 'L' ? 1 : -1;
  int code = 0;
  if (up < 0) code = 1;
  else if (n < 0) code = 2;
  else if (nrhs < 0) code = 3;
  else if (lda < (n > 1 ? n : 1)) code = 5;
  else if (ldb < (n > 1 ? n : 1)) code = 7;
  if (code) {
    call_xerbla("DPOTRS", code);
    return GB_ERR_INVALID_VALUE;
  }
  int st = ensure_init();
  if (st) return st;
  if (n == 0 || nrhs == 0) return GB_SUCCESS;
  return potrs_device(up, n, nrhs, A, lda, B, ldb, stream());
}

}  // extern "C"
