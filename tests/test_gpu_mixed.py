"""Mixed-precision DGESV (FP32 LU + FP64 refinement, GMRES-IR, FP64 fallback).

Bars: backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)
<= n * eps64 for every solve; ITER and the FP32 pivots of the reference's
dsgesv on its golden cases; the ITER codes of the fallback paths (-2 FP32
overflow, -31 no convergence) on the Fortran entry, which keeps the
reference's algorithm; GMRES-IR (device entry) on kappa = 1e8 and 1e12
without falling back to FP64 LU."""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np
import pytest

from conftest import EPS

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import gen_golden as GG  # noqa: E402

from openblas_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


def berr(A, X, B):
    r = np.abs(B - A @ X).max(axis=0)
    den = np.abs(A).sum(axis=1).max() * np.abs(X).max(axis=0) + np.abs(B).max(axis=0)
    return float((r / den).max())


def dsgesv(F, A, B):
    n, nrhs = B.shape
    A = A.copy(order="F")
    X = np.zeros((n, nrhs), order="F")
    ipiv = np.zeros(n, np.int32)
    work = np.zeros((n, nrhs), order="F")
    swork = np.zeros(n * (n + nrhs), np.float32)
    info, it = F.dsgesv(n, nrhs, A, n, ipiv, B, n, X, n, work, swork)
    return info, it, X, ipiv


def test_dsgesv_golden(golden, F, gb_clean):
    for idx, (n, nrhs) in enumerate(GG.DSGESV_CASES):
        A = W.uniform(8400 + idx, (n, n))
        B = W.uniform(8500 + idx, (n, nrhs))
        info, it, X, ipiv = dsgesv(F, A, B)
        assert info == 0
        assert abs(it - int(golden[f"dsgesv_{idx}_iter"])) <= 1, it
        assert np.array_equal(ipiv, golden[f"dsgesv_{idx}_ipiv"])
        assert berr(A, X, B) <= n * EPS
        assert np.abs(X - golden[f"dsgesv_{idx}_x"]).max() <= 1e-10 * np.abs(X).max()


def test_dsgesv_fallback_no_convergence(golden, F, gb_clean):
    n = 60
    A = W.ill_conditioned(8600, n, 12)
    B = W.uniform(8601, (n, 1))
    info, it, X, ipiv = dsgesv(F, A, B)
    assert info == 0 and it == int(golden["dsgesv_ill_iter"]) == -31
    assert np.array_equal(ipiv, golden["dsgesv_ill_ipiv"])
    assert berr(A, X, B) <= n * EPS


def test_dsgesv_overflow_fallback(F, gb_clean):
    n = 40
    A = W.uniform(5, (n, n))
    A[3, 7] = 1e300  # not representable in FP32 -> ITER = -2, FP64 solve
    B = W.uniform(6, (n, 2))
    info, it, X, _ = dsgesv(F, A, B)
    assert info == 0 and it == -2
    assert berr(A, X, B) <= n * EPS


def test_dsgesv_singular(F, gb_clean):
    n = 30
    A = W.uniform(7, (n, n))
    A[:, 11] = 0.0
    B = W.uniform(8, (n, 1))
    info, it, X, _ = dsgesv(F, A, B)
    assert info == 12 and it == -3


@pytest.mark.parametrize("n,nrhs", [(2000, 1), (2000, 64), (3000, 3), (1537, 11)])
def test_dsgesv_uniform(F, gb_clean, n, nrhs):
    A = W.uniform(11, (n, n))
    B = W.uniform(12, (n, nrhs))
    info, it, X, _ = dsgesv(F, A, B)
    assert info == 0 and 0 <= it <= 10, it
    assert berr(A, X, B) <= n * EPS


def _dev_solve(gblib, A, B):
    torch = pytest.importorskip("torch")
    n, nrhs = B.shape
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()   # column-major buffer
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dX = torch.zeros_like(dB)
    dp = torch.zeros(n, dtype=torch.int32, device="cuda")
    it, info = C.c_int(0), C.c_int(0)
    st = gblib.gb_dsgesv_dev(n, nrhs, dA.data_ptr(), n, dp.data_ptr(), dB.data_ptr(), n,
                             dX.data_ptr(), n, C.byref(it), C.byref(info))
    assert st == 0
    return it.value, info.value, dX.cpu().numpy().T.copy(order="F")


@pytest.mark.parametrize("kappa", [4, 8, 12])
def test_gmres_ir_ill_conditioned(gblib, gb_clean, kappa):
    n = 600
    A = W.ill_conditioned(900 + kappa, n, kappa)
    B = W.uniform(901, (n, 2))
    it, info, X = _dev_solve(gblib, A, B)
    assert info == 0
    if kappa == 8:
        assert it >= 100, it  # finished by GMRES-IR, no FP64 LU fallback
    elif kappa == 12:
        # finished by GMRES-IR, or by the FP64-accurate LU fallback (-31)
        assert it >= 100 or it == -31, it
    else:
        assert 0 <= it <= 30
    assert berr(A, X, B) <= n * EPS


def test_device_entry_uniform(gblib, gb_clean):
    n = 1500
    A = W.uniform(21, (n, n))
    B = W.uniform(22, (n, 4))
    it, info, X = _dev_solve(gblib, A, B)
    assert info == 0 and 0 <= it <= 6
    assert berr(A, X, B) <= n * EPS
