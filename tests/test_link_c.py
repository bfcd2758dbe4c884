"""Linking a C program against libgbblas in place of OpenBLAS.

A small C program is compiled against include/gbblas.h and linked with
-lgbblas, as an application would be relinked.  It checks three things:
- the Fortran and CBLAS symbols resolve from C;
- the library's xerbla_ is weak, so an xerbla_ defined by the application
  receives the argument errors (driver/others/xerbla.c declares it weak for
  the same reason);
- quick returns (m = 0, n = 0) succeed with no device.
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
#include "gbblas.h"

static char last_name[16];
static int last_info = -1, calls = 0;

/* the application's own error handler replaces the library's weak one */
int xerbla_(const char *name, const blasint *info, blasint len) {
  size_t n = (size_t)len < sizeof(last_name) - 1 ? (size_t)len : sizeof(last_name) - 1;
  memcpy(last_name, name, n);
  last_name[n] = 0;
  last_info = *info;
  ++calls;
  return 0;
}

int main(void) {
  double a[16] = {0}, b[16] = {0}, c[16] = {0};
  blasint four = 4, three = 3, zero = 0;
  double one = 1.0, nought = 0.0;
  dgemm_("N", "N", &four, &four, &four, &one, a, &three, b, &four, &nought, c, &four);
  if (calls != 1 || last_info != 8 || strncmp(last_name, "DGEMM", 5) != 0) {
    printf("dgemm_: calls %d info %d name '%s'\n", calls, last_info, last_name);
    return 1;
  }
  cblas_dtrsm(CblasColMajor, (enum CBLAS_SIDE)99, CblasLower, CblasNoTrans, CblasNonUnit, 4, 4,
              1.0, a, 4, b, 4);
  if (calls != 2 || last_info != 1 || strncmp(last_name, "DTRSM", 5) != 0) {
    printf("cblas_dtrsm: calls %d info %d name '%s'\n", calls, last_info, last_name);
    return 2;
  }
  int ipiv[4];
  blasint info = 7;
  dgetrf_(&zero, &four, a, &four, ipiv, &info);
  if (info != 0) { printf("dgetrf_ quick return: info %d\n", (int)info); return 3; }
  cblas_dgemm(CblasRowMajor, CblasNoTrans, CblasNoTrans, 0, 4, 4, 1.0, a, 4, b, 4, 0.0, c, 4);
  if (calls != 2) { printf("quick return reported an error\n"); return 4; }
  printf("ok\n");
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_c_program_links_and_overrides_xerbla(tmp_path, gblib):
    libdir = os.path.join(ROOT, "openblas_gb300")
    assert os.path.exists(os.path.join(libdir, "libgbblas.so"))
    src = tmp_path / "app.c"
    exe = tmp_path / "app"
    src.write_text(PROGRAM)
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-I", os.path.join(ROOT, "include"), str(src),
                        "-L", libdir, "-lgbblas", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("ok")
