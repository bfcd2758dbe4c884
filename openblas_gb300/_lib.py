"""Loader and ctypes bindings of libgbblas.so (the CUDA library).

The library must have been built (``python -m openblas_gb300._build`` or
``__graft_entry__.build()``); loading never falls back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
from types import SimpleNamespace

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "libgbblas.so")

_i, _i64, _d, _f, _c, _vp = C.c_int, C.c_int64, C.c_double, C.c_float, C.c_char, C.c_void_p

DEV_SIGS = {
    "gb_set_stream": (_i, [_vp]),
    "gb_get_stream": (_vp, []),
    "gb_synchronize": (_i, []),
    "gb_last_error": (_i, [C.c_char_p, _i]),
    "gb_clear_error": (None, []),
    "gb_last_xerbla": (_i, [C.c_char_p, _i]),
    "gb_set_dgemm_mode": (_i, [_i]),
    "gb_get_dgemm_mode": (_i, []),
    "gb_set_sgemm_mode": (_i, [_i]),
    "gb_get_sgemm_mode": (_i, []),
    "gb_set_ozaki_slices": (_i, [_i]),
    "gb_last_ozaki_slices": (_i, []),
    "gb_last_ozaki_moduli": (_i, []),
    "gb_set_ozaki_modular": (_i, [_i]),
    "gb_version": (C.c_char_p, []),
    "gb_kernel_launches": (C.c_int64, []),
    "gb_profile_enable": (_i, [_i]),
    "gb_profile_kernel_ms": (_d, [C.c_char_p, C.POINTER(_i), _i]),
    "gb_dgemm_dev": (_i, [_c, _c, _i64, _i64, _i64, _d, _vp, _i64, _vp, _i64, _d, _vp, _i64]),
    "gb_dgemm_native_dev": (_i, [_c, _c, _i64, _i64, _i64, _d, _vp, _i64, _vp, _i64, _d, _vp,
                                 _i64]),
    "gb_dgemm_emulated_dev": (_i, [_c, _c, _i64, _i64, _i64, _d, _vp, _i64, _vp, _i64, _d, _vp,
                                   _i64, _i]),
    "gb_sgemm_dev": (_i, [_c, _c, _i64, _i64, _i64, _f, _vp, _i64, _vp, _i64, _f, _vp, _i64]),
    "gb_dtrsm_dev": (_i, [_c, _c, _c, _c, _i64, _i64, _d, _vp, _i64, _vp, _i64]),
    "gb_dsyrk_dev": (_i, [_c, _c, _i64, _i64, _d, _vp, _i64, _d, _vp, _i64]),
    "gb_dtrmm_dev": (_i, [_c, _c, _c, _c, _i64, _i64, _d, _vp, _i64, _vp, _i64]),
    "gb_dsyr2k_dev": (_i, [_c, _c, _i64, _i64, _d, _vp, _i64, _vp, _i64, _d, _vp, _i64]),
    "gb_zgemm_dev": (_i, [_c, _c, _i64, _i64, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _i64]),
    "gb_cgemm_dev": (_i, [_c, _c, _i64, _i64, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _i64]),
    "gb_zgemm3m_dev": (_i, [_c, _c, _i64, _i64, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _i64]),
    "gb_cgemm3m_dev": (_i, [_c, _c, _i64, _i64, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _vp, _i64]),
    "gb_dgemmt_dev": (_i, [_c, _c, _c, _i64, _i64, _d, _vp, _i64, _vp, _i64, _d, _vp, _i64]),
    "gb_dgetrf_dev": (_i, [_i64, _i64, _vp, _i64, _vp, _vp]),
    "gb_dgetrs_dev": (_i, [_c, _i64, _i64, _vp, _i64, _vp, _vp, _i64]),
    "gb_sgetrf_dev": (_i, [_i64, _i64, _vp, _i64, _vp, _vp]),
    "gb_sgetrs_dev": (_i, [_c, _i64, _i64, _vp, _i64, _vp, _vp, _i64]),
    "gb_dlaswp_dev": (_i, [_i64, _vp, _i64, _i64, _i64, _vp, _i64]),
    "gb_dpotrf_dev": (_i, [_c, _i64, _vp, _i64, _vp]),
    "gb_dpotrs_dev": (_i, [_c, _i64, _i64, _vp, _i64, _vp, _i64]),
    "gb_dsposv_dev": (_i, [_c, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, C.POINTER(_i),
                           C.POINTER(_i)]),
    "gb_dgetrf_noalloc_dev": (_i, [_i64, _i64, _vp, _i64, _vp, _vp, _vp]),
    "gb_dsgesv_dev": (_i, [_i64, _i64, _vp, _i64, _vp, _vp, _i64, _vp, _i64, C.POINTER(_i),
                           C.POINTER(_i)]),
}

_cache = {}


def load(path: str | None = None) -> C.CDLL:
    """Load libgbblas.so; raises if it has not been built."""
    path = path or SO
    if path in _cache:
        return _cache[path]
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built; run __graft_entry__.build() first")
    lib = C.CDLL(path, mode=C.RTLD_GLOBAL)
    for name, (res, args) in DEV_SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _cache[path] = lib
    return lib


def fortran(path: str | None = None) -> abi.Fortran:
    """Fortran-ABI wrappers (dgemm_, dgetrf_, ...) over libgbblas."""
    return abi.Fortran(abi.bind(load(path)))


def cblas(path: str | None = None) -> SimpleNamespace:
    return abi.bind(load(path))


def last_error(lib: C.CDLL | None = None) -> tuple[int, str]:
    lib = lib or load()
    buf = C.create_string_buffer(512)
    st = lib.gb_last_error(buf, 512)
    return st, buf.value.decode()


def last_xerbla(lib: C.CDLL | None = None) -> tuple[str, int]:
    lib = lib or load()
    buf = C.create_string_buffer(16)
    info = lib.gb_last_xerbla(buf, 16)
    return buf.value.decode(), info
