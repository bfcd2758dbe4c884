"""GB300 (sm_103a) implementation of OpenBLAS's level-3 BLAS + blocked-LAPACK hot path.

The product is the C-ABI shared library ``libgbblas.so`` (declared in
include/gbblas.h): cblas_dgemm/dgemm_/sgemm_/dtrsm_/dsyrk_/dgetrf_/dgetrs_/
dgesv_/dpotrf_/dlaswp_/dsgesv_/cblas_dgemm_batch plus device-pointer
``gb_*_dev`` variants.  This package builds and loads it and provides the
ctypes bindings used by Python callers.
"""
from ._lib import SO, cblas, fortran, last_error, last_xerbla, load  # noqa: F401

__all__ = ["SO", "load", "fortran", "cblas", "last_error", "last_xerbla"]
