"""C-ABI boundary checks that need no GPU: every symbol declared in
include/*.h is exported, argument errors reach xerbla with the reference's
parameter positions (interface/*.c), LAPACK routines set Info = -position,
and quick returns do not touch the device."""
from __future__ import annotations

import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

import openblas_gb300 as gb
from openblas_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src):
            name = m.group(1)
            start = src.rfind("\n", 0, m.start())
            line = src[start:m.start()]
            if re.search(r"\b(void|int|const char \*|void \*|double|float)\s*\**\s*$", line):
                names.add(name)
    return sorted(names)


def test_exports_every_declared_symbol(gblib):
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(gblib, n)]
    assert not missing, missing


def test_version(gblib):
    assert b"sm_103a" in gblib.gb_version()


def _xerbla(gblib):
    return gb.last_xerbla(gblib)


@pytest.mark.parametrize("args,pos", [
    (("X", "N", 4, 4, 4, 4, 4, 4), 1),
    (("N", "X", 4, 4, 4, 4, 4, 4), 2),
    (("N", "N", -1, 4, 4, 4, 4, 4), 3),
    (("N", "N", 4, -1, 4, 4, 4, 4), 4),
    (("N", "N", 4, 4, -1, 4, 4, 4), 5),
    (("N", "N", 4, 4, 4, 3, 4, 4), 8),
    (("T", "N", 4, 4, 5, 4, 5, 4), 8),
    (("N", "N", 4, 4, 4, 4, 3, 4), 10),
    (("N", "T", 4, 5, 4, 4, 4, 4), 10),
    (("N", "N", 4, 4, 4, 4, 4, 3), 13),
])
def test_dgemm_argument_errors(gblib, F, args, pos):
    ta, tb, m, n, k, lda, ldb, ldc = args
    buf = np.zeros((64, 64), order="F")
    gblib.gb_clear_error()
    F.dgemm(ta, tb, m, n, k, 1.0, buf, lda, buf, ldb, 0.0, buf, ldc)
    name, info = _xerbla(gblib)
    assert name.strip() == "DGEMM" and info == pos


def test_cblas_rowmajor_positions(gblib):
    ns = gb.cblas()
    buf = np.zeros(256)
    gblib.gb_clear_error()
    # row-major A is m x k with lda >= k; the operand swap reports it as B (10)
    ns.cblas_dgemm(abi.CblasRowMajor, abi.CblasNoTrans, abi.CblasNoTrans, 4, 3, 5, 1.0,
                   buf.ctypes.data, 4, buf.ctypes.data, 3, 0.0, buf.ctypes.data, 3)
    assert _xerbla(gblib) == ("DGEMM ", 10)
    gblib.gb_clear_error()
    ns.cblas_sgemm(abi.CblasRowMajor, abi.CblasNoTrans, abi.CblasNoTrans, 4, 3, 5, 1.0,
                   buf.ctypes.data, 4, buf.ctypes.data, 3, 0.0, buf.ctypes.data, 3)
    assert _xerbla(gblib) == ("SGEMM ", 10)
    gblib.gb_clear_error()
    ns.cblas_sgemm(abi.CblasRowMajor, abi.CblasNoTrans, abi.CblasTrans, 4, 3, 5, 1.0,
                   buf.ctypes.data, 5, buf.ctypes.data, 5, 0.0, buf.ctypes.data, 2)
    assert _xerbla(gblib) == ("SGEMM ", 13)  # row-major C is m x n with ldc >= n
    gblib.gb_clear_error()
    ns.cblas_dgemm(77, abi.CblasNoTrans, abi.CblasNoTrans, 4, 3, 5, 1.0, buf.ctypes.data, 4,
                   buf.ctypes.data, 5, 0.0, buf.ctypes.data, 4)
    assert _xerbla(gblib)[1] == 0  # invalid order: xerbla with position 0
    gblib.gb_clear_error()
    ns.cblas_dtrsm(abi.CblasColMajor, 99, abi.CblasLower, abi.CblasNoTrans, abi.CblasNonUnit, 4,
                   4, 1.0, buf.ctypes.data, 4, buf.ctypes.data, 4)
    assert _xerbla(gblib) == ("DTRSM ", 1)
    gblib.gb_clear_error()
    ns.cblas_dsyrk(abi.CblasColMajor, abi.CblasLower, abi.CblasNoTrans, 5, 2, 1.0,
                   buf.ctypes.data, 4, 0.0, buf.ctypes.data, 5)
    assert _xerbla(gblib) == ("DSYRK ", 7)


@pytest.mark.parametrize("args,pos", [
    (("X", "L", "N", "N", 4, 4, 4, 4), 1),
    (("L", "X", "N", "N", 4, 4, 4, 4), 2),
    (("L", "L", "X", "N", 4, 4, 4, 4), 3),
    (("L", "L", "N", "X", 4, 4, 4, 4), 4),
    (("L", "L", "N", "N", -1, 4, 4, 4), 5),
    (("L", "L", "N", "N", 4, -1, 4, 4), 6),
    (("L", "L", "N", "N", 4, 4, 3, 4), 9),
    (("R", "L", "N", "N", 4, 5, 4, 4), 9),
    (("L", "L", "N", "N", 4, 4, 4, 3), 11),
])
def test_dtrsm_argument_errors(gblib, F, args, pos):
    side, uplo, ta, diag, m, n, lda, ldb = args
    buf = np.zeros((64, 64), order="F")
    gblib.gb_clear_error()
    F.dtrsm(side, uplo, ta, diag, m, n, 1.0, buf, lda, buf, ldb)
    assert _xerbla(gblib) == ("DTRSM ", pos)


def test_dsyrk_argument_errors(gblib, F):
    buf = np.zeros((64, 64), order="F")
    for args, pos in [(("X", "N", 4, 4, 4, 4), 1), (("L", "X", 4, 4, 4, 4), 2),
                      (("L", "N", -1, 4, 4, 4), 3), (("L", "N", 4, -1, 4, 4), 4),
                      (("L", "N", 4, 4, 3, 4), 7), (("L", "T", 4, 5, 4, 4), 7),
                      (("L", "N", 4, 4, 4, 3), 10)]:
        uplo, tr, n, k, lda, ldc = args
        gblib.gb_clear_error()
        F.dsyrk(uplo, tr, n, k, 1.0, buf, lda, 0.0, buf, ldc)
        assert _xerbla(gblib) == ("DSYRK ", pos), args


def test_lapack_argument_errors(gblib, F):
    buf = np.zeros((64, 64), order="F")
    piv = np.zeros(64, np.int32)
    assert F.dgetrf(-1, 4, buf, 4, piv) == -1
    assert F.dgetrf(4, -1, buf, 4, piv) == -2
    assert F.dgetrf(4, 4, buf, 3, piv) == -4
    assert _xerbla(gblib) == ("DGETRF", 4)
    assert F.dpotrf("X", 4, buf, 4) == -1
    assert F.dpotrf("L", -2, buf, 4) == -2
    assert F.dpotrf("U", 4, buf, 3) == -4
    assert F.dgesv(-1, 1, buf, 4, piv, buf, 4) == -1
    assert F.dgesv(4, -1, buf, 4, piv, buf, 4) == -2
    assert F.dgesv(4, 1, buf, 3, piv, buf, 4) == -4
    assert F.dgesv(4, 1, buf, 4, piv, buf, 3) == -7
    assert _xerbla(gblib) == ("DGESV", 7)  # interface/lapack/gesv.c:49, no padding
    gblib.gb_clear_error()
    F.dgetrs("X", 4, 1, buf, 4, piv, buf, 4)
    assert _xerbla(gblib) == ("DGETRS", 1)
    F.dgetrs("N", 4, 1, buf, 4, piv, buf, 3)
    assert _xerbla(gblib) == ("DGETRS", 8)


def test_dsgesv_argument_errors(gblib, F):
    buf = np.zeros((64, 64), order="F")
    piv = np.zeros(64, np.int32)
    w = np.zeros(64 * 64)
    sw = np.zeros(64 * 64, np.float32)
    # lapack-netlib/SRC/dsgesv.f:236-249
    for args, pos in [((-1, 1, 4, 4, 4), 1), ((4, -1, 4, 4, 4), 2), ((4, 1, 3, 4, 4), 4),
                      ((4, 1, 4, 3, 4), 7), ((4, 1, 4, 4, 3), 9)]:
        n, nrhs, lda, ldb, ldx = args
        info, it = F.dsgesv(n, nrhs, buf, lda, piv, buf, ldb, buf, ldx, w, sw)
        assert info == -pos and it == 0
        assert _xerbla(gblib) == ("DSGESV", pos)


def test_trmm_syr2k_gemmt_argument_errors(gblib, F):
    buf = np.zeros((64, 64), order="F")
    # interface/trsm.c built as TRMM: the TRSM positions under the name DTRMM
    for args, pos in [(("X", "L", "N", "N", 4, 4, 4, 4), 1), (("L", "X", "N", "N", 4, 4, 4, 4), 2),
                      (("L", "L", "X", "N", 4, 4, 4, 4), 3), (("L", "L", "N", "X", 4, 4, 4, 4), 4),
                      (("L", "L", "N", "N", -1, 4, 4, 4), 5), (("L", "L", "N", "N", 4, -1, 4, 4), 6),
                      (("R", "L", "N", "N", 4, 6, 5, 4), 9), (("L", "L", "N", "N", 4, 4, 4, 3), 11)]:
        side, uplo, ta, diag, m, n, lda, ldb = args
        F.dtrmm(side, uplo, ta, diag, m, n, 1.0, buf, lda, buf, ldb)
        assert _xerbla(gblib) == ("DTRMM ", pos), args
    # interface/syr2k.c:169-175
    for args, pos in [(("X", "N", 4, 2, 4, 4, 4), 1), (("L", "X", 4, 2, 4, 4, 4), 2),
                      (("L", "N", -1, 2, 4, 4, 4), 3), (("L", "N", 4, -1, 4, 4, 4), 4),
                      (("L", "N", 4, 2, 3, 4, 4), 7), (("L", "T", 4, 6, 6, 5, 4), 9),
                      (("U", "N", 4, 2, 4, 4, 3), 12)]:
        uplo, tr, n, k, lda, ldb, ldc = args
        F.dsyr2k(uplo, tr, n, k, 1.0, buf, lda, buf, ldb, 0.0, buf, ldc)
        assert _xerbla(gblib) == ("DSYR2K", pos), args
    # interface/gemmt.c:177-192
    for args, pos in [(("X", "N", "N", 4, 2, 4, 2, 4), 1), (("L", "X", "N", 4, 2, 4, 2, 4), 2),
                      (("L", "N", "X", 4, 2, 4, 2, 4), 3), (("L", "N", "N", -1, 2, 4, 2, 4), 4),
                      (("L", "N", "N", 4, -1, 4, 2, 4), 5), (("L", "N", "N", 4, 2, 3, 2, 4), 8),
                      (("L", "N", "T", 4, 2, 4, 3, 4), 10), (("U", "N", "N", 4, 2, 4, 2, 3), 13)]:
        uplo, ta, tb, m, k, lda, ldb, ldc = args
        F.dgemmt(uplo, ta, tb, m, k, 1.0, buf, lda, buf, ldb, 0.0, buf, ldc)
        assert _xerbla(gblib) == ("DGEMMT ", pos), args  # gemmt.c:44


def test_complex_gemm_argument_errors(gblib, F):
    """interface/gemm.c with COMPLEX: R and C are the conjugate op codes; the
    real GEMM's positions under the names ZGEMM, CGEMM, ZGEMM3M, CGEMM3M."""
    buf = np.zeros((64, 64), np.complex128, order="F")
    bufs = np.zeros((64, 64), np.complex64, order="F")
    cases = [(("X", "N", 4, 4, 4, 4, 4, 4), 1), (("N", "X", 4, 4, 4, 4, 4, 4), 2),
             (("N", "N", -1, 4, 4, 4, 4, 4), 3), (("N", "N", 4, -1, 4, 4, 4, 4), 4),
             (("N", "N", 4, 4, -1, 4, 4, 4), 5), (("C", "N", 4, 4, 5, 4, 5, 4), 8),
             (("R", "N", 4, 4, 4, 3, 4, 4), 8), (("N", "C", 4, 5, 4, 4, 4, 4), 10),
             (("N", "R", 4, 4, 5, 4, 4, 4), 10), (("N", "N", 4, 4, 4, 4, 4, 3), 13)]
    for fn, name, b in (("zgemm", "ZGEMM ", buf), ("cgemm", "CGEMM ", bufs),
                        ("zgemm3m", "ZGEMM3M ", buf), ("cgemm3m", "CGEMM3M ", bufs)):
        for args, pos in cases:
            ta, tb, m, n, k, lda, ldb, ldc = args
            gblib.gb_clear_error()
            getattr(F, fn)(ta, tb, m, n, k, 1.0, b, lda, b, ldb, 0.0, b, ldc)
            assert _xerbla(gblib) == (name, pos), (fn, args)
    # CBLAS: ConjNoTrans/ConjTrans are accepted; row-major swaps the operands
    ns = gb.cblas()
    one = np.array([1.0, 0.0])
    gblib.gb_clear_error()
    ns.cblas_zgemm(101, 114, 113, 4, 4, 4, one.ctypes.data, buf.ctypes.data, 3,
                   buf.ctypes.data, 4, one.ctypes.data, buf.ctypes.data, 4)
    assert _xerbla(gblib) == ("ZGEMM ", 10)  # row-major A (lda 3 < k) is the swapped B
    ns.cblas_zgemm(102, 111, 115, 4, 4, 4, one.ctypes.data, buf.ctypes.data, 4,
                   buf.ctypes.data, 4, one.ctypes.data, buf.ctypes.data, 4)
    assert _xerbla(gblib) == ("ZGEMM ", 2)


def test_dsposv_dpotrs_argument_errors(gblib, F):
    buf = np.zeros((64, 64), order="F")
    w = np.zeros(64 * 64)
    sw = np.zeros(64 * 64, np.float32)
    # lapack-netlib/SRC/dsposv.f:236-251 (UPLO, N, NRHS, LDA, LDB, LDX)
    for args, pos in [(("X", 4, 1, 4, 4, 4), 1), (("L", -1, 1, 4, 4, 4), 2),
                      (("U", 4, -1, 4, 4, 4), 3), (("L", 4, 1, 3, 4, 4), 5),
                      (("L", 4, 1, 4, 3, 4), 7), (("U", 4, 1, 4, 4, 3), 9)]:
        uplo, n, nrhs, lda, ldb, ldx = args
        info, it = F.dsposv(uplo, n, nrhs, buf, lda, buf, ldb, buf, ldx, w, sw)
        assert info == -pos and it == 0
        assert _xerbla(gblib) == ("DSPOSV", pos)
    # lapack-netlib/SRC/dpotrs.f:124-137 (UPLO, N, NRHS, LDA, LDB)
    for args, pos in [(("Q", 4, 1, 4, 4), 1), (("L", -2, 1, 4, 4), 2), (("L", 4, -1, 4, 4), 3),
                      (("U", 4, 1, 2, 4), 5), (("U", 4, 1, 4, 2), 7)]:
        uplo, n, nrhs, lda, ldb = args
        assert F.dpotrs(uplo, n, nrhs, buf, lda, buf, ldb) == -pos
        assert _xerbla(gblib) == ("DPOTRS", pos)
    # quick returns (no device call)
    assert F.dpotrs("L", 0, 3, buf, 4, buf, 4) == 0
    assert F.dpotrs("U", 4, 0, buf, 4, buf, 4) == 0
    assert F.dsposv("L", 0, 1, buf, 4, buf, 4, buf, 4, w, sw) == (0, 0)


def test_quick_returns_do_not_touch_device(gblib, F):
    """m==0/n==0 quick returns happen before any CUDA call, so they succeed on
    a machine without a GPU (interface/gemm.c:494, getrf.c:83, potrf.c:104)."""
    buf = np.zeros((4, 4), order="F")
    piv = np.zeros(4, np.int32)
    gblib.gb_clear_error()
    F.dgemm("N", "N", 0, 4, 4, 1.0, buf, 4, buf, 4, 0.0, buf, 4)
    F.dtrsm("L", "L", "N", "N", 4, 0, 1.0, buf, 4, buf, 4)
    F.dsyrk("L", "N", 0, 4, 1.0, buf, 4, 0.0, buf, 4)
    assert F.dgetrf(0, 4, buf, 4, piv) == 0
    assert F.dpotrf("L", 0, buf, 4) == 0
    assert F.dgesv(0, 1, buf, 4, piv, buf, 4) == 0
    F.dlaswp(4, buf, 4, 1, 4, piv, 0)
    assert gb.last_error(gblib)[0] == 0


def test_xerbla_message_format(gblib, capfd):
    """driver/others/xerbla.c:58: ' ** On entry to %6s parameter number %2d ...'
    -- %6s pads short names and keeps long ones whole; a Fortran caller's name
    carries no terminator and is bounded by the hidden length."""
    info = C.c_int(3)
    gblib.xerbla_(b"DGEMM ", C.byref(info), 6)
    gblib.xerbla_(b"ZGEMM3M ", C.byref(info), 8)
    gblib.xerbla_(b"DGEMM_BATCH ", C.byref(info), 12)
    gblib.xerbla_(b"DGETRFXYZ", C.byref(info), 6)
    out = capfd.readouterr().out
    assert " ** On entry to DGEMM  parameter number  3 had an illegal value" in out
    assert " ** On entry to ZGEMM3M  parameter number  3 had an illegal value" in out
    assert " ** On entry to DGEMM_BATCH  parameter number  3 had an illegal value" in out
    assert " ** On entry to DGETRF parameter number  3 had an illegal value" in out


def test_dgemm_batch_argument_errors(gblib):
    """interface/gemm_batch.c:195-283: every group is checked before any group
    runs; errors are reported as DGEMM_BATCH (gemm_batch.c:44) with the GEMM
    positions (row-major swaps the operands first), and an unknown order
    with position 0.  All pointers are null: nothing may run."""
    from openblas_gb300 import abi

    def iarr(v):
        return (C.c_int * len(v))(*v)

    def call(order, ta, tb, ms, ns, ks, lda, ldb, ldc):
        g = len(ms)
        nulls = (C.c_void_p * g)()
        gblib.gb_clear_error()
        gblib.cblas_dgemm_batch(order, iarr(ta), iarr(tb), iarr(ms), iarr(ns), iarr(ks),
                                (C.c_double * g)(*[1.0] * g), nulls, iarr(lda), nulls,
                                iarr(ldb), (C.c_double * g)(*[0.0] * g), nulls, iarr(ldc),
                                g, iarr([1] * g))
        name, info = gb.last_xerbla(gblib)
        return name.strip(), info

    N, T = abi.CblasNoTrans, abi.CblasTrans
    col, row = abi.CblasColMajor, abi.CblasRowMajor
    # the second group is bad: the first, valid one must not have run
    assert call(col, [N, N], [N, N], [4, 4], [4, 4], [4, 4], [4, 4], [4, 4], [4, 3]) == \
        ("DGEMM_BATCH", 13)
    assert call(col, [N, 7], [N, N], [4, 4], [4, 4], [4, 4], [4, 4], [4, 4], [4, 4]) == \
        ("DGEMM_BATCH", 1)
    assert call(col, [N], [T], [4], [5], [4], [4], [4], [4]) == ("DGEMM_BATCH", 10)
    assert call(col, [N], [N], [4], [4], [-1], [4], [4], [4]) == ("DGEMM_BATCH", 5)
    # row-major A (m x k, lda >= k) with lda < k: the swapped B operand's ldb (10)
    assert call(row, [N], [N], [4], [5], [6], [5], [5], [5]) == ("DGEMM_BATCH", 10)
    assert call(999, [N], [N], [4], [4], [4], [4], [4], [4]) == ("DGEMM_BATCH", 0)
