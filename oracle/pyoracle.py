"""ctypes front-end of the oracle library (oracle/liborc.so).

TEST INFRASTRUCTURE ONLY: used by the tests, the smoke check and the
CPU-baseline leg of bench.py, as the reference results and the CPU baseline.  Same argument
order as the Fortran ABI wrappers in openblas_gb300.abi.Fortran so a test can
run one case through either.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_i, _d, _f, _c, _vp = C.c_int, C.c_double, C.c_float, C.c_char, C.c_void_p
_pi = C.POINTER(C.c_int)

_SIGS = {
    "orc_set_threads": (None, [_i]),
    "orc_get_threads": (_i, []),
    "orc_dgemm": (None, [_c, _c, _i, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i]),
    "orc_sgemm": (None, [_c, _c, _i, _i, _i, _f, _vp, _i, _vp, _i, _f, _vp, _i]),
    "orc_dgemm_dd": (None, [_c, _c, _i, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i]),
    "orc_dgemm_absbound": (None, [_c, _c, _i, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i, _vp, _i]),
    "orc_dtrsm": (None, [_c, _c, _c, _c, _i, _i, _d, _vp, _i, _vp, _i]),
    "orc_dsyrk": (None, [_c, _c, _i, _i, _d, _vp, _i, _d, _vp, _i]),
    "orc_dlaswp": (None, [_i, _vp, _i, _i, _i, _vp, _i]),
    "orc_dgetrf": (_i, [_i, _i, _vp, _i, _vp]),
    "orc_sgetrf": (_i, [_i, _i, _vp, _i, _vp]),
    "orc_dgetrs": (_i, [_c, _i, _i, _vp, _i, _vp, _vp, _i]),
    "orc_sgetrs": (_i, [_c, _i, _i, _vp, _i, _vp, _vp, _i]),
    "orc_dgesv": (_i, [_i, _i, _vp, _i, _vp, _vp, _i]),
    "orc_dpotrf": (_i, [_c, _i, _vp, _i]),
    "orc_dsgesv": (_i, [_i, _i, _vp, _i, _vp, _vp, _i, _vp, _i, _pi]),
    "orc_dlange_inf": (_d, [_i, _i, _vp, _i]),
    "orc_dpotrs": (_i, [_c, _i, _i, _vp, _i, _vp, _i]),
    "orc_dtrmm": (None, [_c, _c, _c, _c, _i, _i, _d, _vp, _i, _vp, _i]),
    "orc_dsyr2k": (None, [_c, _c, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i]),
    "orc_dgemmt": (None, [_c, _c, _c, _i, _i, _d, _vp, _i, _vp, _i, _d, _vp, _i]),
    "orc_dsposv": (_i, [_c, _i, _i, _vp, _i, _vp, _i, _vp, _i, _pi]),
    "orc_zgemm": (None, [_c, _c, _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _vp, _i]),
    "orc_cgemm": (None, [_c, _c, _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _vp, _i]),
    "orc_zgemm3m": (None, [_c, _c, _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _vp, _i]),
    "orc_cgemm3m": (None, [_c, _c, _i, _i, _i, _vp, _vp, _i, _vp, _i, _vp, _vp, _i]),
    "orc_batch": (None, [_vp, _i]),
}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        so = _build.SO
        if not os.path.exists(so):
            so = _build.build()
        _lib = C.CDLL(so)
        for name, (res, args) in _SIGS.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args
    return _lib


def _p(a):
    if a is None:
        return None
    if a.ndim > 1 and not a.flags["F_CONTIGUOUS"]:
        raise ValueError("column-major (Fortran-ordered) array required")
    return a.ctypes.data_as(_vp)


def _ch(s: str) -> bytes:
    return s.encode()[:1]


def set_threads(n: int) -> None:
    lib().orc_set_threads(n)


def get_threads() -> int:
    return lib().orc_get_threads()


def dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    lib().orc_dgemm(_ch(ta), _ch(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc)


def sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    lib().orc_sgemm(_ch(ta), _ch(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc)


def dgemm_dd(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    lib().orc_dgemm_dd(_ch(ta), _ch(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc)


def dgemm_absbound(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    G = np.zeros((m, n), order="F")
    lib().orc_dgemm_absbound(_ch(ta), _ch(tb), m, n, k, alpha, _p(A), lda, _p(B), ldb, beta,
                             _p(Cm), ldc, _p(G), max(m, 1))
    return G


def dtrsm(side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb):
    lib().orc_dtrsm(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, alpha, _p(A), lda, _p(B), ldb)


def dsyrk(uplo, trans, n, k, alpha, A, lda, beta, Cm, ldc):
    lib().orc_dsyrk(_ch(uplo), _ch(trans), n, k, alpha, _p(A), lda, beta, _p(Cm), ldc)


def dlaswp(n, A, lda, k1, k2, ipiv, incx):
    lib().orc_dlaswp(n, _p(A), lda, k1, k2, _p(ipiv), incx)


def dgetrf(m, n, A, lda, ipiv) -> int:
    return lib().orc_dgetrf(m, n, _p(A), lda, _p(ipiv))


def sgetrf(m, n, A, lda, ipiv) -> int:
    return lib().orc_sgetrf(m, n, _p(A), lda, _p(ipiv))


def dgetrs(trans, n, nrhs, A, lda, ipiv, B, ldb) -> int:
    return lib().orc_dgetrs(_ch(trans), n, nrhs, _p(A), lda, _p(ipiv), _p(B), ldb)


def dgesv(n, nrhs, A, lda, ipiv, B, ldb) -> int:
    return lib().orc_dgesv(n, nrhs, _p(A), lda, _p(ipiv), _p(B), ldb)


def dpotrf(uplo, n, A, lda) -> int:
    return lib().orc_dpotrf(_ch(uplo), n, _p(A), lda)


def dsgesv(n, nrhs, A, lda, ipiv, B, ldb, X, ldx):
    it = C.c_int(0)
    info = lib().orc_dsgesv(n, nrhs, _p(A), lda, _p(ipiv), _p(B), ldb, _p(X), ldx, C.byref(it))
    return info, it.value


def dtrmm(side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb):
    lib().orc_dtrmm(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, alpha, _p(A), lda, _p(B), ldb)


def dsyr2k(uplo, trans, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    lib().orc_dsyr2k(_ch(uplo), _ch(trans), n, k, alpha, _p(A), lda, _p(B), ldb, beta, _p(Cm), ldc)


def _complex_gemm(name, real, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    al = np.array([complex(alpha).real, complex(alpha).imag], dtype=real)
    be = np.array([complex(beta).real, complex(beta).imag], dtype=real)
    getattr(lib(), name)(_ch(ta), _ch(tb), m, n, k, _p(al), _p(A), lda, _p(B), ldb, _p(be),
                         _p(Cm), ldc)


def zgemm(*args):
    _complex_gemm("orc_zgemm", np.float64, *args)


def cgemm(*args):
    _complex_gemm("orc_cgemm", np.float32, *args)


def zgemm3m(*args):
    _complex_gemm("orc_zgemm3m", np.float64, *args)


def cgemm3m(*args):
    _complex_gemm("orc_cgemm3m", np.float32, *args)


def dgemmt(uplo, ta, tb, m, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
    lib().orc_dgemmt(_ch(uplo), _ch(ta), _ch(tb), m, k, alpha, _p(A), lda, _p(B), ldb, beta,
                     _p(Cm), ldc)


def dpotrs(uplo, n, nrhs, A, lda, B, ldb) -> int:
    return lib().orc_dpotrs(_ch(uplo), n, nrhs, _p(A), lda, _p(B), ldb)


def dsposv(uplo, n, nrhs, A, lda, B, ldb, X, ldx):
    it = C.c_int(0)
    info = lib().orc_dsposv(_ch(uplo), n, nrhs, _p(A), lda, _p(B), ldb, _p(X), ldx, C.byref(it))
    return info, it.value


def dlange_inf(m, n, A, lda) -> float:
    return lib().orc_dlange_inf(m, n, _p(A), lda)
