"""DTRMM, DSYR2K and DGEMMT on the GPU (interface/trsm.c as TRMM,
interface/syr2k.c, interface/gemmt.c): OpenBLAS golden outputs for every
side/uplo/trans/diag combination and the alpha/beta edge values, larger
shapes against the oracle with the DMMCH-style bound, the emulated-FP64
mode, and CBLAS row-major calls against their column-major equivalents.
The triangle a routine does not own must come back bit for bit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from openblas_gb300 import workloads as W
from tests.conftest import dmmch_ratio
from tests.golden import gen_golden as GG

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _other(uplo, X):
    return np.triu(X, 1) if uplo == "L" else np.tril(X, -1)


def test_dtrmm_golden(golden, F, gb_clean):
    idx = 0
    for (m, n) in GG.TRSM_SHAPES:
        for side in "LR":
            for uplo in "UL":
                for ta in "NT":
                    for diag in "UN":
                        for alpha in GG.TRSM_ALPHA:
                            A, B = GG.trmm_operands(idx, side, uplo, m, n)
                            F.dtrmm(side, uplo, ta, diag, m, n, alpha, A, A.shape[0], B, m)
                            ref = golden[f"dtrmm_{idx}"]
                            scale = max(1.0, np.abs(ref).max())
                            assert np.max(np.abs(B - ref)) <= 4 * A.shape[0] * EPS * scale, (
                                idx, side, uplo, ta, diag, alpha)
                            idx += 1


def test_dsyr2k_golden(golden, F, gb_clean):
    idx = 0
    for (n, k) in GG.SYRK_SHAPES:
        for uplo in "UL":
            for tr in "NT":
                for (alpha, beta) in GG.SYRK_AB:
                    ra, ca = (n, k) if tr == "N" else (k, n)
                    A = W.uniform(9700 + idx, (ra, ca))
                    B = W.uniform(9800 + idx, (ra, ca))
                    Cm = W.uniform(9900 + idx, (n, n))
                    C0 = Cm.copy(order="F")
                    F.dsyr2k(uplo, tr, n, k, alpha, A, ra, B, ra, beta, Cm, n)
                    ref = golden[f"dsyr2k_{idx}"]
                    assert np.max(np.abs(Cm - ref)) <= 8 * (k + 2) * EPS * max(1, np.abs(ref).max())
                    assert np.array_equal(_other(uplo, Cm), _other(uplo, C0))
                    idx += 1


def test_dgemmt_golden(golden, F, gb_clean):
    idx = 0
    for (m, k) in GG.GEMMT_SHAPES:
        for uplo in "UL":
            for ta in "NT":
                for tb in "NT":
                    for (alpha, beta) in GG.GEMMT_AB:
                        A = W.uniform(10000 + idx, (m, k) if ta == "N" else (k, m))
                        B = W.uniform(10100 + idx, (k, m) if tb == "N" else (m, k))
                        Cm = W.uniform(10200 + idx, (m, m))
                        C0 = Cm.copy(order="F")
                        F.dgemmt(uplo, ta, tb, m, k, alpha, A, A.shape[0], B, B.shape[0],
                                 beta, Cm, m)
                        ref = golden[f"dgemmt_{idx}"]
                        assert np.max(np.abs(Cm - ref)) <= 4 * (k + 2) * EPS * max(1, np.abs(ref).max())
                        assert np.array_equal(_other(uplo, Cm), _other(uplo, C0))
                        idx += 1


@pytest.mark.parametrize("side,uplo,ta,diag", [("L", "L", "N", "N"), ("L", "U", "T", "U"),
                                               ("R", "L", "T", "N"), ("R", "U", "N", "U")])
def test_dtrmm_large_vs_oracle(orc, F, gb_clean, side, uplo, ta, diag):
    m, n = 700, 900
    na = m if side == "L" else n
    A = W.uniform(9100, (na, na))
    B = W.uniform(9101, (m, n))
    B0, Bo = B.copy(order="F"), B.copy(order="F")
    F.dtrmm(side, uplo, ta, diag, m, n, -1.25, A, na, B, m)
    orc.dtrmm(side, uplo, ta, diag, m, n, -1.25, A, na, Bo, m)
    T = np.tril(A) if uplo == "L" else np.triu(A)
    if diag == "U":
        np.fill_diagonal(T, 1.0)
    oT = np.abs(T.T if ta == "T" else T)
    G = 1.25 * (oT @ np.abs(B0) if side == "L" else np.abs(B0) @ oT)
    assert dmmch_ratio(B, Bo, G, na) <= 2 * (na + 2)


@pytest.mark.parametrize("uplo,tr", [("L", "N"), ("U", "T")])
def test_dsyr2k_large_vs_oracle(orc, F, gb_clean, uplo, tr):
    n, k = 1100, 300
    ra, ca = (n, k) if tr == "N" else (k, n)
    A, B = W.uniform(9200, (ra, ca)), W.uniform(9201, (ra, ca))
    Cm = W.uniform(9202, (n, n))
    C0, Co = Cm.copy(order="F"), Cm.copy(order="F")
    F.dsyr2k(uplo, tr, n, k, 0.6, A, ra, B, ra, 1.4, Cm, n)
    orc.dsyr2k(uplo, tr, n, k, 0.6, A, ra, B, ra, 1.4, Co, n)
    oA, oB = (A, B) if tr == "N" else (A.T, B.T)
    G = 0.6 * (np.abs(oA) @ np.abs(oB).T + np.abs(oB) @ np.abs(oA).T) + 1.4 * np.abs(C0)
    tri = np.tril if uplo == "L" else np.triu
    assert dmmch_ratio(tri(Cm), tri(Co), tri(G), 2 * k) <= 2 * (2 * k + 2)
    assert np.array_equal(_other(uplo, Cm), _other(uplo, C0))


@pytest.mark.parametrize("mode", [0, 1])
def test_dgemmt_large_vs_oracle(orc, F, gblib, gb_clean, mode):
    """Native FP64 and, in DGEMM mode 'emulated', the Ozaki GEMM restricted
    to the triangle (tiles wholly in the other triangle are skipped)."""
    m, k = 1300, 700
    A, B = W.uniform(9300, (k, m)), W.uniform(9301, (k, m))   # op(A) = A^T, op(B) = B
    Cm = W.uniform(9302, (m, m))
    C0, Co = Cm.copy(order="F"), Cm.copy(order="F")
    gblib.gb_set_dgemm_mode(mode)
    try:
        F.dgemmt("U", "T", "N", m, k, 0.9, A, k, B, k, -0.3, Cm, m)
    finally:
        gblib.gb_set_dgemm_mode(0)
    orc.dgemmt("U", "T", "N", m, k, 0.9, A, k, B, k, -0.3, Co, m)
    G = 0.9 * np.abs(A).T @ np.abs(B) + 0.3 * np.abs(C0)
    assert dmmch_ratio(np.triu(Cm), np.triu(Co), np.triu(G), k) <= 2 * (k + 2)
    assert np.array_equal(_other("U", Cm), _other("U", C0))


def test_cblas_row_major_forms(gblib, gb_clean):
    """Row-major CBLAS calls equal the column-major call on the transposed
    data (interface/trsm.c, syr2k.c, gemmt.c row-major mappings)."""
    from openblas_gb300 import cblas
    ns = cblas()
    m, n, k = 37, 29, 23
    # dtrmm: row-major B (m x n) = alpha * A(m x m, lower) * B
    A = np.ascontiguousarray(W.uniform(9400, (m, m)))
    B = np.ascontiguousarray(W.uniform(9401, (m, n)))
    ref = 1.5 * np.tril(A) @ B
    ns.cblas_dtrmm(101, 141, 122, 111, 131, m, n, 1.5, A.ctypes.data, m, B.ctypes.data, n)
    assert np.max(np.abs(B - ref)) <= 64 * m * EPS * np.abs(ref).max()
    # dsyr2k: row-major C (n x n, upper) = A B^T + B A^T + 0.5 C
    A = np.ascontiguousarray(W.uniform(9402, (n, k)))
    B = np.ascontiguousarray(W.uniform(9403, (n, k)))
    Cr = np.ascontiguousarray(W.uniform(9404, (n, n)))
    ref = A @ B.T + B @ A.T + 0.5 * Cr
    low = np.tril(Cr, -1).copy()
    ns.cblas_dsyr2k(101, 121, 111, n, k, 1.0, A.ctypes.data, k, B.ctypes.data, k, 0.5,
                    Cr.ctypes.data, n)
    assert np.max(np.abs(np.triu(Cr) - np.triu(ref))) <= 64 * k * EPS * np.abs(ref).max()
    assert np.array_equal(np.tril(Cr, -1), low)
    # dgemmt: row-major C (m x m, lower) = A(m x k) B^T(k x m) + C
    A = np.ascontiguousarray(W.uniform(9405, (m, k)))
    B = np.ascontiguousarray(W.uniform(9406, (m, k)))
    Cr = np.ascontiguousarray(W.uniform(9407, (m, m)))
    ref = A @ B.T + Cr
    up = np.triu(Cr, 1).copy()
    ns.cblas_dgemmt(101, 122, 111, 112, m, k, 1.0, A.ctypes.data, k, B.ctypes.data, k, 1.0,
                    Cr.ctypes.data, m)
    assert np.max(np.abs(np.tril(Cr) - np.tril(ref))) <= 64 * k * EPS * np.abs(ref).max()
    assert np.array_equal(np.triu(Cr, 1), up)


def test_device_entries(gblib, gb_clean):
    torch = pytest.importorskip("torch")
    m, k = 640, 200
    A = W.uniform(9500, (m, k))
    Cm = W.uniform(9501, (m, m))
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(Cm.T)).cuda()
    assert gblib.gb_dsyr2k_dev(b"L", b"N", m, k, 1.0, dA.data_ptr(), m, dA.data_ptr(), m, 0.0,
                               dC.data_ptr(), m) == 0
    assert gblib.gb_synchronize() == 0  # the call is stream-ordered on the library's stream
    got = dC.cpu().numpy().T
    ref = 2.0 * A @ A.T
    assert np.max(np.abs(np.tril(got) - np.tril(ref))) <= 64 * k * EPS * np.abs(ref).max()
    assert np.array_equal(np.triu(got, 1), np.triu(Cm, 1))
