"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; the rest run on CPU."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "openblas_golden.npz")
EPS = np.finfo(np.float64).eps


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN, allow_pickle=False)


@pytest.fixture(scope="session")
def orc():
    from oracle import build as obuild
    obuild.build()
    from oracle import pyoracle
    return pyoracle


@pytest.fixture(scope="session")
def gblib():
    from openblas_gb300 import _build
    _build.build()
    import openblas_gb300 as gb
    return gb.load()


@pytest.fixture(scope="session")
def F(gblib):
    import openblas_gb300 as gb
    return gb.fortran()


@pytest.fixture
def gb_clean(gblib):
    gblib.gb_clear_error()
    yield gblib
    import openblas_gb300 as gb
    st, msg = gb.last_error(gblib)
    assert st in (0, 1), f"library error after test: {msg}"


def dmmch_ratio(Cgot, Cref, G, k):
    """max |Cgot-Cref| / (eps * G), the DMMCH test ratio of ctest/c_dblat3c.c:2956
    with the denominator guarded where G == 0 (then both must be exact)."""
    d = np.abs(np.asarray(Cgot, dtype=np.float64) - np.asarray(Cref, dtype=np.float64))
    G = np.asarray(G, dtype=np.float64)
    bad = (G == 0) & (d != 0)
    if bad.any():
        return np.inf
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(G > 0, d / (EPS * np.where(G > 0, G, 1.0)), 0.0)
    return float(r.max()) if r.size else 0.0


def complex_op(X, rows, cols, code):
    """op(X) of the stored complex matrix X[:rows, :cols] for op code N, T,
    R (conjugate) or C (conjugate transpose)."""
    X = X[:rows, :cols]
    if code in "TC":
        X = X.T
    if code in "RC":
        X = X.conj()
    return X


def zgemm_ratio(Cgot, Cref, A, B, C0, m, n, k, ta, tb, alpha, beta, eps, normwise=False):
    """DMMCH-style ratio for a complex GEMM: max |Cgot - Cref| / (eps G) with
    G = |alpha| |op(A)| |op(B)| + |beta| |C0| (moduli), componentwise, or
    with G replaced by its maximum (normwise: the 3M products and the
    emulated-FP64 engine are bounded normwise, not per element)."""
    ra, ca = (m, k) if ta in "NR" else (k, m)
    rb, cb = (k, n) if tb in "NR" else (n, k)
    oA = np.abs(complex_op(A, ra, ca, ta)).astype(np.float64)
    oB = np.abs(complex_op(B, rb, cb, tb)).astype(np.float64)
    G = abs(alpha) * (oA @ oB) if k > 0 else np.zeros((m, n))
    if beta != 0:
        G = G + abs(beta) * np.abs(C0[:m, :n]).astype(np.float64)
    if normwise:
        G = np.full_like(G, G.max() if G.size else 0.0)
    d = np.abs(np.asarray(Cgot[:m, :n], dtype=np.complex128) -
               np.asarray(Cref[:m, :n], dtype=np.complex128))
    if ((G == 0) & (d != 0)).any() or np.isnan(d).any():
        return np.inf
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(G > 0, d / (eps * np.where(G > 0, G, 1.0)), 0.0)
    return float(r.max()) if r.size else 0.0
