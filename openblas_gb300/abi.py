"""ctypes declarations of the BLAS/LAPACK C ABI (cblas_* and Fortran-77 ``name_``).

``bind(lib, prefix)`` returns a namespace of typed callables for every symbol
of the drop-in boundary.  It binds libgbblas.so (prefix "") -- this is the
ctypes stub a Python caller would use -- and, in the golden-vector generator,
an OpenBLAS build whose symbols carry a prefix.

Fortran conventions: every argument by pointer, characters as ``char*``
(hidden string lengths are not read by either library), ``blasint`` = int32,
LAPACK routines return int (interface/lapack/*.c), BLAS routines void.
"""
from __future__ import annotations

import ctypes as C
from types import SimpleNamespace

import numpy as np

# CBLAS enum values (cblas.h:62-66)
CblasRowMajor, CblasColMajor = 101, 102
CblasNoTrans, CblasTrans, CblasConjTrans, CblasConjNoTrans = 111, 112, 113, 114
CblasUpper, CblasLower = 121, 122
CblasNonUnit, CblasUnit = 131, 132
CblasLeft, CblasRight = 141, 142

_i = C.c_int
_pi = C.POINTER(C.c_int)
_pd = C.POINTER(C.c_double)
_pf = C.POINTER(C.c_float)
_pc = C.c_char_p
_d = C.c_double
_f = C.c_float
_vp = C.c_void_p

FORTRAN_SIGS = {
    # BLAS level 3 (interface/gemm.c:181, trsm.c:114, syrk.c:96)
    "dgemm_": (None, [_pc, _pc, _pi, _pi, _pi, _pd, _vp, _pi, _vp, _pi, _pd, _vp, _pi]),
    "sgemm_": (None, [_pc, _pc, _pi, _pi, _pi, _pf, _vp, _pi, _vp, _pi, _pf, _vp, _pi]),
    "dtrsm_": (None, [_pc, _pc, _pc, _pc, _pi, _pi, _pd, _vp, _pi, _vp, _pi]),
    "dsyrk_": (None, [_pc, _pc, _pi, _pi, _pd, _vp, _pi, _pd, _vp, _pi]),
    "dtrmm_": (None, [_pc, _pc, _pc, _pc, _pi, _pi, _pd, _vp, _pi, _vp, _pi]),
    "dsyr2k_": (None, [_pc, _pc, _pi, _pi, _pd, _vp, _pi, _vp, _pi, _pd, _vp, _pi]),
    "dgemmt_": (None, [_pc, _pc, _pc, _pi, _pi, _pd, _vp, _pi, _vp, _pi, _pd, _vp, _pi]),
    # complex GEMM (interface/gemm.c with COMPLEX / GEMM3M): alpha, beta -> (re, im)
    "zgemm_": (None, [_pc, _pc, _pi, _pi, _pi, _vp, _vp, _pi, _vp, _pi, _vp, _vp, _pi]),
    "cgemm_": (None, [_pc, _pc, _pi, _pi, _pi, _vp, _vp, _pi, _vp, _pi, _vp, _vp, _pi]),
    "zgemm3m_": (None, [_pc, _pc, _pi, _pi, _pi, _vp, _vp, _pi, _vp, _pi, _vp, _vp, _pi]),
    "cgemm3m_": (None, [_pc, _pc, _pi, _pi, _pi, _vp, _vp, _pi, _vp, _pi, _vp, _vp, _pi]),
    # LAPACK (interface/lapack/*.c)
    "dgetrf_": (_i, [_pi, _pi, _vp, _pi, _vp, _pi]),
    "dgetrs_": (_i, [_pc, _pi, _pi, _vp, _pi, _vp, _vp, _pi, _pi]),
    "dgesv_": (_i, [_pi, _pi, _vp, _pi, _vp, _vp, _pi, _pi]),
    "dpotrf_": (_i, [_pc, _pi, _vp, _pi, _pi]),
    "dlaswp_": (_i, [_pi, _vp, _pi, _pi, _pi, _vp, _pi]),
    "dsgesv_": (_i, [_pi, _pi, _vp, _pi, _vp, _vp, _pi, _vp, _pi, _vp, _vp, _pi, _pi]),
    "dpotrs_": (_i, [_pc, _pi, _pi, _vp, _pi, _vp, _pi, _pi]),
    "dsposv_": (_i, [_pc, _pi, _pi, _vp, _pi, _vp, _pi, _vp, _pi, _vp, _vp, _pi, _pi]),
    "sgetrf_": (_i, [_pi, _pi, _vp, _pi, _vp, _pi]),
}

CBLAS_SIGS = {
    "cblas_dgemm": (None, [_i, _i, _i, _i, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i]),
    "cblas_sgemm": (None, [_i, _i, _i, _i, _i, _i, _f, _vp, _i, _vp, _i, _f, _vp, _i]),
    "cblas_dtrsm": (None, [_i, _i, _i, _i, _i, _i, _i, _d, _vp, _i, _vp, _i]),
    "cblas_dsyrk": (None, [_i, _i, _i, _i, _i, _d, _vp, _i, _d, _vp, _i]),
    "cblas_dtrmm": (None, [_i, _i, _i, _i, _i, _i, _i, _d, _vp, _i, _vp, _i]),
    "cblas_dsyr2k": (None, [_i, _i, _i, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i]),
    "cblas_dgemmt": (None, [_i, _i, _i, _i, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i]),
    "cblas_zgemm": (None, [_i, _i, _i, _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _vp, _i]),
    "cblas_cgemm": (None, [_i, _i, _i, _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _vp, _i]),
    "cblas_zgemm3m": (None, [_i, _i, _i, _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _vp, _i]),
    "cblas_cgemm3m": (None, [_i, _i, _i, _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _vp, _i]),
    "cblas_dgemm_batch": (None, [_i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                 _vp, _vp, _i, _vp]),
}


def _ptr(a) -> C.c_void_p:
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    if isinstance(a, np.ndarray):
        if a.ndim > 1 and not a.flags["F_CONTIGUOUS"]:
            raise ValueError("column-major (Fortran-ordered) array required")
        return a.ctypes.data_as(C.c_void_p)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    raise TypeError(type(a))


def bind(lib: C.CDLL, prefix: str = "", symbols=None) -> SimpleNamespace:
    """Attach argtypes/restype to ``lib``'s ABI symbols; missing ones are skipped."""
    ns = SimpleNamespace()
    sigs = dict(FORTRAN_SIGS)
    sigs.update(CBLAS_SIGS)
    for name, (res, args) in sigs.items():
        if symbols is not None and name not in symbols:
            continue
        try:
            fn = getattr(lib, prefix + name)
        except AttributeError:
            continue
        fn.restype = res
        fn.argtypes = args
        setattr(ns, name, fn)
    ns._lib = lib
    return ns


class Fortran:
    """Numpy-friendly wrappers over a bound ABI namespace (column-major arrays)."""

    def __init__(self, ns: SimpleNamespace):
        self.ns = ns

    @staticmethod
    def _c(ch: str) -> bytes:
        return ch.encode()

    def dgemm(self, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
        self.ns.dgemm_(self._c(ta), self._c(tb), C.byref(_i(m)), C.byref(_i(n)), C.byref(_i(k)),
                       C.byref(_d(alpha)), _ptr(A), C.byref(_i(lda)), _ptr(B), C.byref(_i(ldb)),
                       C.byref(_d(beta)), _ptr(Cm), C.byref(_i(ldc)))

    def _complex_gemm(self, fn, real, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
        al = np.array([complex(alpha).real, complex(alpha).imag], dtype=real)
        be = np.array([complex(beta).real, complex(beta).imag], dtype=real)
        fn(self._c(ta), self._c(tb), C.byref(_i(m)), C.byref(_i(n)), C.byref(_i(k)),
           al.ctypes.data_as(C.c_void_p), _ptr(A), C.byref(_i(lda)), _ptr(B), C.byref(_i(ldb)),
           be.ctypes.data_as(C.c_void_p), _ptr(Cm), C.byref(_i(ldc)))

    def zgemm(self, *args):
        self._complex_gemm(self.ns.zgemm_, np.float64, *args)

    def cgemm(self, *args):
        self._complex_gemm(self.ns.cgemm_, np.float32, *args)

    def zgemm3m(self, *args):
        self._complex_gemm(self.ns.zgemm3m_, np.float64, *args)

    def cgemm3m(self, *args):
        self._complex_gemm(self.ns.cgemm3m_, np.float32, *args)

    def sgemm(self, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
        self.ns.sgemm_(self._c(ta), self._c(tb), C.byref(_i(m)), C.byref(_i(n)), C.byref(_i(k)),
                       C.byref(_f(alpha)), _ptr(A), C.byref(_i(lda)), _ptr(B), C.byref(_i(ldb)),
                       C.byref(_f(beta)), _ptr(Cm), C.byref(_i(ldc)))

    def dtrsm(self, side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb):
        self.ns.dtrsm_(self._c(side), self._c(uplo), self._c(ta), self._c(diag), C.byref(_i(m)),
                       C.byref(_i(n)), C.byref(_d(alpha)), _ptr(A), C.byref(_i(lda)), _ptr(B),
                       C.byref(_i(ldb)))

    def dsyrk(self, uplo, trans, n, k, alpha, A, lda, beta, Cm, ldc):
        self.ns.dsyrk_(self._c(uplo), self._c(trans), C.byref(_i(n)), C.byref(_i(k)),
                       C.byref(_d(alpha)), _ptr(A), C.byref(_i(lda)), C.byref(_d(beta)), _ptr(Cm),
                       C.byref(_i(ldc)))

    def dgetrf(self, m, n, A, lda, ipiv) -> int:
        info = _i(0)
        self.ns.dgetrf_(C.byref(_i(m)), C.byref(_i(n)), _ptr(A), C.byref(_i(lda)), _ptr(ipiv),
                        C.byref(info))
        return info.value

    def sgetrf(self, m, n, A, lda, ipiv) -> int:
        info = _i(0)
        self.ns.sgetrf_(C.byref(_i(m)), C.byref(_i(n)), _ptr(A), C.byref(_i(lda)), _ptr(ipiv),
                        C.byref(info))
        return info.value

    def dgetrs(self, trans, n, nrhs, A, lda, ipiv, B, ldb) -> int:
        info = _i(0)
        self.ns.dgetrs_(self._c(trans), C.byref(_i(n)), C.byref(_i(nrhs)), _ptr(A),
                        C.byref(_i(lda)), _ptr(ipiv), _ptr(B), C.byref(_i(ldb)), C.byref(info))
        return info.value

    def dgesv(self, n, nrhs, A, lda, ipiv, B, ldb) -> int:
        info = _i(0)
        self.ns.dgesv_(C.byref(_i(n)), C.byref(_i(nrhs)), _ptr(A), C.byref(_i(lda)), _ptr(ipiv),
                       _ptr(B), C.byref(_i(ldb)), C.byref(info))
        return info.value

    def dpotrf(self, uplo, n, A, lda) -> int:
        info = _i(0)
        self.ns.dpotrf_(self._c(uplo), C.byref(_i(n)), _ptr(A), C.byref(_i(lda)), C.byref(info))
        return info.value

    def dtrmm(self, side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb):
        self.ns.dtrmm_(self._c(side), self._c(uplo), self._c(ta), self._c(diag), C.byref(_i(m)),
                       C.byref(_i(n)), C.byref(_d(alpha)), _ptr(A), C.byref(_i(lda)), _ptr(B),
                       C.byref(_i(ldb)))

    def dsyr2k(self, uplo, trans, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
        self.ns.dsyr2k_(self._c(uplo), self._c(trans), C.byref(_i(n)), C.byref(_i(k)),
                        C.byref(_d(alpha)), _ptr(A), C.byref(_i(lda)), _ptr(B), C.byref(_i(ldb)),
                        C.byref(_d(beta)), _ptr(Cm), C.byref(_i(ldc)))

    def dgemmt(self, uplo, ta, tb, m, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
        self.ns.dgemmt_(self._c(uplo), self._c(ta), self._c(tb), C.byref(_i(m)), C.byref(_i(k)),
                        C.byref(_d(alpha)), _ptr(A), C.byref(_i(lda)), _ptr(B), C.byref(_i(ldb)),
                        C.byref(_d(beta)), _ptr(Cm), C.byref(_i(ldc)))

    def dpotrs(self, uplo, n, nrhs, A, lda, B, ldb) -> int:
        info = _i(0)
        self.ns.dpotrs_(self._c(uplo), C.byref(_i(n)), C.byref(_i(nrhs)), _ptr(A),
                        C.byref(_i(lda)), _ptr(B), C.byref(_i(ldb)), C.byref(info))
        return info.value

    def dsposv(self, uplo, n, nrhs, A, lda, B, ldb, X, ldx, work, swork):
        it = _i(0)
        info = _i(0)
        self.ns.dsposv_(self._c(uplo), C.byref(_i(n)), C.byref(_i(nrhs)), _ptr(A),
                        C.byref(_i(lda)), _ptr(B), C.byref(_i(ldb)), _ptr(X), C.byref(_i(ldx)),
                        _ptr(work), _ptr(swork), C.byref(it), C.byref(info))
        return info.value, it.value

    def dlaswp(self, n, A, lda, k1, k2, ipiv, incx):
        self.ns.dlaswp_(C.byref(_i(n)), _ptr(A), C.byref(_i(lda)), C.byref(_i(k1)),
                        C.byref(_i(k2)), _ptr(ipiv), C.byref(_i(incx)))

    def dsgesv(self, n, nrhs, A, lda, ipiv, B, ldb, X, ldx, work, swork):
        it = _i(0)
        info = _i(0)
        self.ns.dsgesv_(C.byref(_i(n)), C.byref(_i(nrhs)), _ptr(A), C.byref(_i(lda)), _ptr(ipiv),
                        _ptr(B), C.byref(_i(ldb)), _ptr(X), C.byref(_i(ldx)), _ptr(work),
                        _ptr(swork), C.byref(it), C.byref(info))
        return info.value, it.value
