// Host/device operand binding for the blocking (host-pointer) entry points.
#pragma once

#include <new>

#include "gb_internal.h"

namespace gb {

// A column-major rows x cols matrix passed by the caller.  If the pointer
// is device memory it is used in place with the caller's leading dimension;
// otherwise a compact device copy (ld = rows) is staged through the stream.
struct Operand {
  void *user = nullptr;
  int64_t rows = 0, cols = 0, ld = 0;
  size_t esize = 8;
  void *dev = nullptr;
  int64_t dld = 0;
  bool staged = false;
  Scratch buf;

  Operand(const void *p, int64_t r, int64_t c, int64_t l, size_t es)
      : user(const_cast<void *>(p)), rows(r), cols(c), ld(l), esize(es) {}

  int bind(bool copy_in, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) {
      dev = user;
      dld = ld > 0 ? ld : 1;
      return GB_SUCCESS;
    }
    if (is_device_pointer(user)) {
      dev = user;
      dld = ld;
      return GB_SUCCESS;
    }
    buf.~Scratch();
    new (&buf) Scratch((size_t)rows * cols * esize, s);
    if (!buf.p) return GB_ERR_ALLOC;
    dev = buf.p;
    dld = rows;
    staged = true;
    if (copy_in) return stage_in(dev, user, ld, rows, cols, esize, s);
    return GB_SUCCESS;
  }
  int unbind(cudaStream_t s) {
    if (!staged) return GB_SUCCESS;
    return stage_out(user, dev, ld, rows, cols, esize, s);
  }
  template <class T>
  T *d() const { return reinterpret_cast<T *>(dev); }
};

// Finish a blocking call: wait for the stream and surface kernel errors.
int finish_blocking(cudaStream_t s);

// Fortran character argument, upper-cased (TOUPPER in common.h).
inline char upch(const char *c) {
  char x = c ? *c : 0;
  return (x >= 'a' && x <= 'z') ? (char)(x - 32) : x;
}
inline char upch(char x) { return (x >= 'a' && x <= 'z') ? (char)(x - 32) : x; }

// GEMM argument checks in the order of interface/gemm.c:274-286 (real and
// COMPLEX builds alike); returns the xerbla parameter position or 0.  Op
// codes: bit 0 set for a transposed operand (T, and C for complex).
inline int gemm_check(int transa, int transb, int64_t m, int64_t n, int64_t k, int64_t lda,
                      int64_t ldb, int64_t ldc) {
  const int64_t nrowa = (transa & 1) ? k : m;
  const int64_t nrowb = (transb & 1) ? n : k;
  int info = 0;
  if (ldc < m) info = 13;
  if (ldb < nrowb) info = 10;
  if (lda < nrowa) info = 8;
  if (k < 0) info = 5;
  if (n < 0) info = 4;
  if (m < 0) info = 3;
  if (transb < 0) info = 2;
  if (transa < 0) info = 1;
  return info;
}

// Records the argument error and calls xerbla_ (which may be overridden).
void call_xerbla(const char *name, int info);
void record_xerbla(const char *name, int info);

}  // namespace gb
