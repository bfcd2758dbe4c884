"""GEMMs split into blocks of C (openblas_gb300/csrc/gemm_blocks.h).

Several launches put a row or column count of C on gridDim.y, which is capped
at 65535.  So a GEMM whose m or n exceeds 2^20 runs as a sequence of GEMMs,
each on a block of C of at most 2^20 rows and columns.  The offsets of the
blocks' op(A) rows, op(B) columns and C entries are plain C++ in that
header.  Here g++ compiles them with a reference column-major GEMM standing in
for the device engines.  The program checks the blocked result bit for bit
against one call over the whole of C:
- all four transpose pairs;
- padded leading dimensions;
- extents that divide m and n, extents that leave ragged edges, and extents
  larger than the matrix.
It also checks that the first failing block's status is returned.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include <vector>
#include "gemm_blocks.h"

// C = alpha op(A) op(B) + beta C, column-major, k summed in order.
static void ref_gemm(int ta, int tb, long m, long n, long k, double alpha, const double *A,
                     long lda, const double *B, long ldb, double beta, double *C, long ldc) {
  for (long j = 0; j < n; ++j)
    for (long i = 0; i < m; ++i) {
      double acc = 0.0;
      for (long p = 0; p < k; ++p) {
        const double a = ta ? A[p + i * lda] : A[i + p * lda];
        const double b = tb ? B[j + p * ldb] : B[p + j * ldb];
        acc += a * b;
      }
      C[i + j * ldc] = alpha * acc + beta * C[i + j * ldc];
    }
}

static double val(long s) {
  unsigned long x = (unsigned long)s * 6364136223846793005ul + 1442695040888963407ul;
  return (double)((x >> 33) % 2001) / 1000.0 - 1.0;
}

int main() {
  const long m = 23, n = 17, k = 9, pad = 3;
  int bad = 0;
  for (int ta = 0; ta < 2; ++ta)
    for (int tb = 0; tb < 2; ++tb) {
      const long ra = ta ? k : m, ca = ta ? m : k, rb = tb ? n : k, cb = tb ? k : n;
      const long lda = ra + pad, ldb = rb + pad, ldc = m + pad;
      std::vector<double> A(lda * ca), B(ldb * cb), C0(ldc * n);
      for (size_t i = 0; i < A.size(); ++i) A[i] = val(i + 1);
      for (size_t i = 0; i < B.size(); ++i) B[i] = val(i + 5000);
      for (size_t i = 0; i < C0.size(); ++i) C0[i] = val(i + 9000);
      std::vector<double> Cfull = C0;
      ref_gemm(ta, tb, m, n, k, 1.5, A.data(), lda, B.data(), ldb, -0.5, Cfull.data(), ldc);
      for (long ext : {1L, 4L, 5L, 17L, 23L, 64L}) {
        std::vector<double> C = C0;
        long calls = 0;
        const int st = gb::gemm_over_blocks(
            ta, tb, m, n, A.data(), lda, B.data(), ldb, C.data(), ldc, ext,
            [&](long mb, long nb, const double *Ai, const double *Bj, double *Cij) {
              if (mb < 1 || nb < 1 || mb > ext || nb > ext) return 9;
              ++calls;
              ref_gemm(ta, tb, mb, nb, k, 1.5, Ai, lda, Bj, ldb, -0.5, Cij, ldc);
              return 0;
            });
        const long want = ((m + ext - 1) / ext) * ((n + ext - 1) / ext);
        if (st != 0 || calls != want || memcmp(C.data(), Cfull.data(), C.size() * 8) != 0) {
          printf("ta %d tb %d extent %ld: status %d, %ld calls of %ld, results %s\n", ta, tb, ext,
                 st, calls, want,
                 memcmp(C.data(), Cfull.data(), C.size() * 8) ? "differ" : "equal");
          ++bad;
        }
      }
    }
  // the first failing block's status comes back and no later block runs
  long calls = 0;
  std::vector<double> A(100), B(100), C(100);
  const int st = gb::gemm_over_blocks(0, 0, 10L, 10L, A.data(), 10L, B.data(), 10L, C.data(),
                                      10L, 3L,
                                      [&](long, long, const double *, const double *, double *) {
                                        return ++calls == 2 ? 5 : 0;
                                      });
  if (st != 5 || calls != 2) { printf("failure: status %d after %ld calls\n", st, calls); ++bad; }
  if (bad) return 1;
  printf("ok\n");
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_blocked_gemm_matches_one_call(tmp_path):
    src = tmp_path / "gemm_blocks_check.cpp"
    exe = tmp_path / "gemm_blocks_check"
    src.write_text(PROGRAM)
    inc = os.path.join(ROOT, "openblas_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", inc, str(src), "-o", str(exe)],
                   check=True, capture_output=True, timeout=120)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"
