"""DPOTRS and the mixed-precision Cholesky solve DSPOSV on the GPU.

dpotrs_ (lapack-netlib/SRC/dpotrs.f) against OpenBLAS golden solutions;
dsposv_ (lapack-netlib/SRC/dsposv.f) against OpenBLAS's ITER codes and
solutions, its FP64 fallbacks (FP32 Cholesky failure: ITER=-3; matrix not
positive definite: info), the untouched A on the FP32 path, and large
sizes through both Fortran and device entries by backward error.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from openblas_gb300 import workloads as W
from tests.golden import gen_golden as GG

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def berr(A, X, B):
    """max over columns of ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)."""
    R = B - A @ X
    an = np.abs(A).sum(axis=1).max()
    num = np.abs(R).max(axis=0)
    den = an * np.abs(X).max(axis=0) + np.abs(B).max(axis=0)
    return float((num / den).max())


def dsposv(F, uplo, A, B):
    n, nrhs = B.shape
    X = np.zeros((n, nrhs), order="F")
    work = np.zeros((n, nrhs), order="F")
    swork = np.zeros(n * (n + nrhs), np.float32)
    info, it = F.dsposv(uplo, n, nrhs, A, n, B, n, X, n, work, swork)
    return info, it, X


def test_dpotrs_golden(golden, F, gb_clean):
    for idx, (uplo, n, nrhs) in enumerate(GG.DPOTRS_CASES):
        A = W.spd(8800 + idx, n)
        assert F.dpotrf(uplo, n, A, n) == 0
        B = W.uniform(8810 + idx, (n, nrhs))
        assert F.dpotrs(uplo, n, nrhs, A, n, B, n) == 0
        ref = golden[f"dpotrs_{idx}_x"]
        assert np.max(np.abs(B - ref)) <= 64 * n * EPS * np.abs(ref).max(), (uplo, n, nrhs)


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_dpotrs_large(F, gb_clean, uplo):
    n, nrhs = 1800, 9
    A0 = W.spd(8840, n)
    A = A0.copy(order="F")
    assert F.dpotrf(uplo, n, A, n) == 0
    B = W.uniform(8841, (n, nrhs))
    X = B.copy(order="F")
    assert F.dpotrs(uplo, n, nrhs, A, n, X, n) == 0
    assert berr(A0, X, B) <= n * EPS


def test_dsposv_golden(golden, F, gb_clean):
    for idx, (uplo, n, nrhs) in enumerate(GG.DSPOSV_CASES):
        A0 = W.spd(8900 + idx, n)
        A = A0.copy(order="F")
        B = W.uniform(8910 + idx, (n, nrhs))
        info, it, X = dsposv(F, uplo, A, B)
        assert info == 0
        assert abs(it - int(golden[f"dsposv_{idx}_iter"])) <= 1, it
        assert np.array_equal(A, A0)  # the FP32 path leaves A as it was
        assert berr(A0, X, B) <= n * EPS
        ref = golden[f"dsposv_{idx}_x"]
        assert np.abs(X - ref).max() <= 1e-10 * np.abs(ref).max()


def test_dsposv_fp32_cholesky_failure_falls_back(golden, F, gb_clean):
    """An SPD matrix with kappa = 1e10: the FP32 Cholesky fails (ITER = -3,
    as in OpenBLAS) and the FP64 DPOTRF/DPOTRS fallback solves it."""
    n = 60
    A0 = W.spd_ill_conditioned(8920, n, 10)
    A = A0.copy(order="F")
    B = W.uniform(8921, (n, 1))
    info, it, X = dsposv(F, "L", A, B)
    assert info == int(golden["dsposv_ill_info"]) == 0
    assert it == int(golden["dsposv_ill_iter"]) == -3
    assert berr(A0, X, B) <= n * EPS
    Lg = np.tril(A)
    assert np.abs(A0 - Lg @ Lg.T).max() <= 1e-12  # A now holds the FP64 factor


def test_dsposv_not_positive_definite(golden, F, gb_clean):
    n = 30
    A = W.spd(8930, n)
    A[17, 17] = -1.0
    B = W.uniform(8931, (n, 1))
    info, it, _ = dsposv(F, "L", A, B)
    assert info == int(golden["dsposv_npd_info"]) == 18
    assert it == int(golden["dsposv_npd_iter"]) == -3


def test_dsposv_overflow_fallback(F, gb_clean):
    n = 40
    A0 = W.spd(8950, n)
    A0[5, 5] = 1e300  # not representable in FP32 -> ITER = -2, FP64 solve
    A = A0.copy(order="F")
    B = W.uniform(8951, (n, 2))
    info, it, X = dsposv(F, "U", A, B)
    assert info == 0 and it == -2
    assert berr(A0, X, B) <= n * EPS


@pytest.mark.parametrize("uplo,n,nrhs", [("L", 2500, 1), ("U", 2500, 4), ("L", 1900, 13)])
def test_dsposv_large(F, gb_clean, uplo, n, nrhs):
    """Blocked FP32 Cholesky (tensor-core trailing updates at these sizes),
    chained solves on the mirrored factor, FP64 refinement."""
    A0 = W.spd(8960 + n, n)
    A = A0.copy(order="F")
    B = W.uniform(8961 + n, (n, nrhs))
    info, it, X = dsposv(F, uplo, A, B)
    assert info == 0 and 0 <= it <= 10, it
    assert np.array_equal(A, A0)
    assert berr(A0, X, B) <= n * EPS


def test_dsposv_device_entry(gblib, gb_clean):
    torch = pytest.importorskip("torch")
    n, nrhs = 3000, 2
    A0 = W.spd(8970, n)
    B = W.uniform(8971, (n, nrhs))
    dA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()   # column-major buffer
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dX = torch.zeros_like(dB)
    it, info = C.c_int(0), C.c_int(0)
    st = gblib.gb_dsposv_dev(b"L", n, nrhs, dA.data_ptr(), n, dB.data_ptr(), n, dX.data_ptr(),
                             n, C.byref(it), C.byref(info))
    assert st == 0 and info.value == 0 and 0 <= it.value <= 10
    X = dX.cpu().numpy().T.copy(order="F")
    assert berr(A0, X, B) <= n * EPS
