"""GPU parity of the level-3 BLAS entry points against the oracle and the
OpenBLAS golden vectors.  GEMM/TRSM/SYRK use the DMMCH-style bound of
ctest/c_dblat3c.c:2956: |C - Cref| <= c * eps * (|alpha||A||B| + |beta||C|),
with c = 2(k+2) (both results carry <= (k+2) eps rounding)."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

from conftest import EPS, dmmch_ratio

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import gen_golden as GG  # noqa: E402

import openblas_gb300 as gb  # noqa: E402
from openblas_gb300 import abi  # noqa: E402
from openblas_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


def test_dgemm_golden_cases(golden, orc, F, gb_clean):
    idx = 0
    for (m, n, k) in GG.GEMM_SHAPES:
        for (alpha, beta) in GG.GEMM_AB:
            for ta in "NT":
                for tb in "NT":
                    A, B, Cm = W.gemm_operands(GG.gemm_case_seed(idx), m, n, k, ta, tb, pad=3)
                    C0 = Cm.copy(order="F")
                    if beta == 0.0:
                        Cm[:m, :n] = np.nan
                    F.dgemm(ta, tb, m, n, k, alpha, A, A.shape[0], B, B.shape[0], beta, Cm,
                            Cm.shape[0])
                    G = orc.dgemm_absbound(ta, tb, m, n, k, alpha, A, A.shape[0], B, B.shape[0],
                                           beta, C0, C0.shape[0])
                    assert not np.isnan(Cm[:m, :n]).any(), idx
                    r = dmmch_ratio(Cm[:m, :n], golden[f"dgemm_{idx}"], G, k)
                    assert r <= 2 * (k + 2), (idx, m, n, k, ta, tb, alpha, beta, r)
                    assert np.array_equal(Cm[m:, :], C0[m:, :])  # padding untouched
                    idx += 1


def test_dgemm_c1_1024(golden, F, gb_clean):
    """1024^3 NN alpha=1.5 beta=0.5 -- the reference's CPU-runnable case."""
    A, B, Cm = W.gemm_operands(42, 1024, 1024, 1024)
    F.dgemm("N", "N", 1024, 1024, 1024, 1.5, A, 1024, B, 1024, 0.5, Cm, 1024)
    G = 1.5 * np.abs(A) @ np.abs(B) + 0.5 * np.abs(W.gemm_operands(42, 1024, 1024, 1024)[2])
    assert np.allclose(Cm.sum(axis=0), golden["dgemm_c1_colsum"], rtol=0,
                       atol=2 * 1026 * EPS * G.sum(axis=0).max())
    r = dmmch_ratio(Cm[::37, ::41], golden["dgemm_c1_sample"], G[::37, ::41], 1024)
    assert r <= 2 * 1026


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_dgemm_padded_lda_vs_oracle(orc, F, gb_clean, ta, tb):
    m, n, k = 1000, 777, 613
    A, B, Cm = W.gemm_operands(91, m, n, k, ta, tb, pad=8)
    C0, Co = Cm.copy(order="F"), Cm.copy(order="F")
    F.dgemm(ta, tb, m, n, k, -0.75, A, A.shape[0], B, B.shape[0], 1.25, Cm, Cm.shape[0])
    orc.dgemm(ta, tb, m, n, k, -0.75, A, A.shape[0], B, B.shape[0], 1.25, Co, Co.shape[0])
    G = orc.dgemm_absbound(ta, tb, m, n, k, -0.75, A, A.shape[0], B, B.shape[0], 1.25, C0,
                           C0.shape[0])
    assert dmmch_ratio(Cm[:m], Co[:m], G, k) <= 2 * (k + 2)
    assert np.array_equal(Cm[m:], C0[m:])


def test_dgemm_rowmajor_cblas(gb_clean):
    ns = gb.cblas()
    m, n, k = 37, 29, 41
    A = np.ascontiguousarray(W.uniform(5, (m, k)))   # row-major m x k
    B = np.ascontiguousarray(W.uniform(6, (k, n)))
    C = np.ascontiguousarray(W.uniform(7, (m, n)))
    ref = 0.5 * A @ B + 2.0 * C
    ns.cblas_dgemm(abi.CblasRowMajor, abi.CblasNoTrans, abi.CblasNoTrans, m, n, k, 0.5,
                   A.ctypes.data, k, B.ctypes.data, n, 2.0, C.ctypes.data, n)
    assert np.max(np.abs(C - ref)) <= 4 * (k + 2) * EPS * (np.abs(A) @ np.abs(B) + 2).max()


@pytest.mark.parametrize("mode", [0, 1])  # native FP64, emulated FP64
def test_svd_reconstruction_rowmajor(gblib, gb_clean, mode):
    """The reference's utest/test_kernel_regress.c check:
    - a 100 x 100 matrix of uniform [0, 10) values is factored by an SVD on the host;
    - it is rebuilt as (U S) Vt by a row-major cblas_dgemm;
    - the Frobenius norm of the difference must stay below 1e-10."""
    ns = gb.cblas()
    N = 100
    M = W.uniform(4242, (N, N), 0.0, 10.0)
    u, s, vt = np.linalg.svd(M)
    us = np.ascontiguousarray(u * s)      # row-major U diag(s)
    vt = np.ascontiguousarray(vt)
    X = np.zeros((N, N))                  # row-major result
    gblib.gb_set_dgemm_mode(mode)
    try:
        ns.cblas_dgemm(abi.CblasRowMajor, abi.CblasNoTrans, abi.CblasNoTrans, N, N, N, 1.0,
                       us.ctypes.data, N, vt.ctypes.data, N, 0.0, X.ctypes.data, N)
    finally:
        gblib.gb_set_dgemm_mode(0)
    assert np.linalg.norm(X - M) < 1e-10


@pytest.mark.parametrize("side,uplo,trans", [
    ("L", "L", "N"), ("L", "U", "T"), ("R", "L", "T"), ("R", "U", "N")])
def test_dtrsm_rowmajor_cblas(gb_clean, side, uplo, trans):
    """Row-major cblas_dtrsm on row-major data (interface/trsm.c:315-351 maps
    it to the column-major solve with m and n swapped, side and uplo flipped):
    X = alpha * op(A)^-1 B (left) or alpha * B op(A)^-1 (right)."""
    ns = gb.cblas()
    m, n, alpha = 70, 45, -0.75
    na = m if side == "L" else n
    L = W.trsm_lower(9100 + na, na)
    A = np.ascontiguousarray(L if uplo == "L" else L.T)      # row-major triangle
    B = np.ascontiguousarray(W.uniform(9200 + na, (m, n)))
    opA = A.T if trans == "T" else A
    tri = np.tril(opA) if (uplo == "L") == (trans == "N") else np.triu(opA)
    X = alpha * (np.linalg.solve(tri, B) if side == "L" else np.linalg.solve(tri.T, B.T).T)
    ns.cblas_dtrsm(abi.CblasRowMajor, abi.CblasLeft if side == "L" else abi.CblasRight,
                   abi.CblasLower if uplo == "L" else abi.CblasUpper,
                   abi.CblasTrans if trans == "T" else abi.CblasNoTrans, abi.CblasNonUnit,
                   m, n, alpha, A.ctypes.data, na, B.ctypes.data, n)
    assert np.max(np.abs(B - X)) <= 64 * na * EPS * max(1.0, np.abs(X).max())


@pytest.mark.parametrize("uplo,trans", [("U", "N"), ("L", "T")])
def test_dsyrk_rowmajor_cblas(gb_clean, uplo, trans):
    """Row-major cblas_dsyrk (interface/syrk.c:309-335 flips uplo and trans):
    the stored triangle of C becomes alpha op(A) op(A)^T + beta C and the
    other triangle is left as it was."""
    ns = gb.cblas()
    n, k, alpha, beta = 60, 33, 1.25, 0.5
    A = np.ascontiguousarray(W.uniform(9300, (n, k) if trans == "N" else (k, n)))
    C0 = np.ascontiguousarray(W.uniform(9301, (n, n)))
    C = C0.copy()
    opA = A if trans == "N" else A.T
    full = alpha * opA @ opA.T + beta * C0
    ns.cblas_dsyrk(abi.CblasRowMajor, abi.CblasUpper if uplo == "U" else abi.CblasLower,
                   abi.CblasNoTrans if trans == "N" else abi.CblasTrans, n, k, alpha,
                   A.ctypes.data, A.shape[1], beta, C.ctypes.data, n)
    keep = np.triu(np.ones((n, n), bool)) if uplo == "U" else np.tril(np.ones((n, n), bool))
    assert np.max(np.abs(C[keep] - full[keep])) <= 4 * (k + 2) * EPS * (abs(alpha) * k + beta)
    assert np.array_equal(C[~keep], C0[~keep])


def test_dgemm_device_pointers(orc, gblib, gb_clean):
    torch = pytest.importorskip("torch")
    m, n, k = 300, 257, 190
    A, B, Cm = W.gemm_operands(13, m, n, k, "T", "N", pad=8)
    dA = torch.from_numpy(A.T.copy()).cuda()  # row-major copy of the column-major buffer
    dB = torch.from_numpy(B.T.copy()).cuda()
    dC = torch.from_numpy(Cm.T.copy()).cuda()
    st = gblib.gb_dgemm_native_dev(b"T", b"N", m, n, k, 0.5, dA.data_ptr(), A.shape[0],
                                   dB.data_ptr(), B.shape[0], -1.0, dC.data_ptr(), Cm.shape[0])
    assert st == 0
    assert gblib.gb_synchronize() == 0
    got = dC.cpu().numpy().T
    Co = Cm.copy(order="F")
    orc.dgemm("T", "N", m, n, k, 0.5, A, A.shape[0], B, B.shape[0], -1.0, Co, Co.shape[0])
    G = orc.dgemm_absbound("T", "N", m, n, k, 0.5, A, A.shape[0], B, B.shape[0], -1.0, Cm,
                           Cm.shape[0])
    assert dmmch_ratio(got[:m], Co[:m], G, k) <= 2 * (k + 2)


def test_sgemm(golden, F, gb_clean):
    A, B, Cm = W.gemm_operands(77, 35, 33, 64, "N", "T", dtype=np.float32)
    C0 = Cm.copy(order="F")
    F.sgemm("N", "T", 35, 33, 64, 0.7, A, 35, B, 33, 1.3, Cm, 35)
    G = 0.7 * np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64)).T + 1.3 * np.abs(C0)
    feps = np.finfo(np.float32).eps
    assert np.max(np.abs(Cm - golden["sgemm_0"]) / (feps * G)) <= 2 * 66


def test_sgemm_large(F, gb_clean):
    m, n, k = 1536, 1100, 700
    A, B, Cm = W.gemm_operands(78, m, n, k, "T", "N", dtype=np.float32)
    ref = 1.0 * A.astype(np.float64).T @ B.astype(np.float64) + 0.5 * Cm.astype(np.float64)
    G = np.abs(A.astype(np.float64)).T @ np.abs(B.astype(np.float64)) + 0.5 * np.abs(Cm)
    F.sgemm("T", "N", m, n, k, 1.0, A, k, B, k, 0.5, Cm, m)
    feps = np.finfo(np.float32).eps
    assert np.max(np.abs(Cm - ref) / (feps * G)) <= (k + 2)


@pytest.fixture
def sgemm_tensor(gblib):
    gblib.gb_set_sgemm_mode(2)   # GB_SGEMM_TENSOR
    yield
    gblib.gb_set_sgemm_mode(0)


def _sgemm_ref(ta, tb, alpha, A, B, beta, C0, m, n, k):
    a = A.astype(np.float64)[:m if ta == "N" else k, :k if ta == "N" else m]
    b = B.astype(np.float64)[:k if tb == "N" else n, :n if tb == "N" else k]
    oa = a if ta == "N" else a.T
    ob = b if tb == "N" else b.T
    c0 = C0.astype(np.float64)[:m, :n]
    ref = alpha * oa @ ob + beta * c0
    G = abs(alpha) * np.abs(oa) @ np.abs(ob) + abs(beta) * np.abs(c0)
    return ref, G


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_sgemm_tensor_cores(F, gb_clean, sgemm_tensor, ta, tb):
    """FP32 GEMM through the bf16x3 tensor-core form: ragged tiles (m, n, k not
    multiples of 128, 256, 64), padded leading dimensions, alpha/beta; the
    DMMCH-style ratio stays within the FP32 GEMM bound k + 2."""
    m, n, k = 1100, 1300, 333
    A, B, Cm = W.gemm_operands(79, m, n, k, ta, tb, pad=5, dtype=np.float32)
    C0 = Cm.copy(order="F")
    F.sgemm(ta, tb, m, n, k, -0.75, A, A.shape[0], B, B.shape[0], 1.25, Cm, Cm.shape[0])
    ref, G = _sgemm_ref(ta, tb, -0.75, A, B, 1.25, C0, m, n, k)
    feps = np.finfo(np.float32).eps
    assert np.max(np.abs(Cm[:m, :n] - ref) / (feps * G)) <= k + 2
    assert np.array_equal(Cm[m:], C0[m:])          # padding rows untouched


@pytest.mark.parametrize("alpha,beta,shape", [
    (-1.0, 1.0, (5000, 2900, 256)),   # the LU trailing update C - A B; 40 x 12 tiles, 3+ per CTA
    (0.5, 0.5, (1100, 1300, 333)),
    (2.0, -2.0, (4100, 1030, 200)),   # 33 x 5 tiles with ragged edges
])
def test_sgemm_tensor_many_tiles(F, gb_clean, sgemm_tensor, alpha, beta, shape):
    """More tiles than SMs (each persistent CTA cycles both TMEM accumulators
    several times), ragged edges, beta = +-alpha as in the LU update: every
    tile and the padding rows come out within the FP32 GEMM bound."""
    m, n, k = shape
    A, B, Cm = W.gemm_operands(81, m, n, k, "N", "N", pad=3, dtype=np.float32)
    C0 = Cm.copy(order="F")
    F.sgemm("N", "N", m, n, k, alpha, A, A.shape[0], B, B.shape[0], beta, Cm, Cm.shape[0])
    ref, G = _sgemm_ref("N", "N", alpha, A, B, beta, C0, m, n, k)
    feps = np.finfo(np.float32).eps
    assert np.max(np.abs(Cm[:m, :n] - ref) / (feps * G)) <= k + 2
    assert np.array_equal(Cm[m:], C0[m:])


def test_sgemm_tensor_update_specials(F, gb_clean, sgemm_tensor):
    """The LU-style update C - A B: rows and columns holding Inf/NaN go to the
    FP32 fixup, and an Inf already in C propagates."""
    m, n, k = 1200, 1100, 96
    A, B, Cm = W.gemm_operands(82, m, n, k, dtype=np.float32)
    A[5, 3] = np.inf
    B[7, 900] = np.nan
    Cm[600, 20] = -np.inf
    C0 = Cm.copy(order="F")
    F.sgemm("N", "N", m, n, k, -1.0, A, m, B, k, 1.0, Cm, m)
    with np.errstate(invalid="ignore"):
        ref = C0.astype(np.float64) - A.astype(np.float64) @ B.astype(np.float64)
    assert np.array_equal(np.isnan(Cm), np.isnan(ref))
    assert np.array_equal(np.isposinf(Cm), np.isposinf(ref))
    assert np.array_equal(np.isneginf(Cm), np.isneginf(ref))
    fin = np.isfinite(ref)
    G = np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64)) + np.abs(C0)
    feps = np.finfo(np.float32).eps
    with np.errstate(invalid="ignore"):
        assert np.max(np.abs(Cm[fin] - ref[fin]) / (feps * G[fin])) <= k + 2


def test_sgemm_tensor_beta_zero_and_specials(F, gb_clean, sgemm_tensor):
    """beta = 0 overwrites C without reading it (NaN in C is not propagated);
    Inf in A propagates as in an FP32 product."""
    m, n, k = 700, 520, 130
    A, B, Cm = W.gemm_operands(80, m, n, k, dtype=np.float32)
    Cm[:] = np.nan
    A[3, 7] = np.inf
    F.sgemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, Cm, m)
    with np.errstate(invalid="ignore"):
        ref = A.astype(np.float64) @ B.astype(np.float64)
    fin = np.isfinite(ref)
    assert np.array_equal(np.isposinf(Cm), np.isposinf(ref))
    assert np.array_equal(np.isneginf(Cm), np.isneginf(ref))
    G = np.abs(A[np.isfinite(A).all(axis=1)].astype(np.float64)) @ np.abs(B.astype(np.float64))
    rows = np.isfinite(A).all(axis=1)
    feps = np.finfo(np.float32).eps
    assert np.max(np.abs(Cm[rows] - ref[rows]) / (feps * G)) <= k + 2
    assert fin[rows].all()


def test_dtrsm_golden_cases(golden, F, gb_clean):
    idx = 0
    for (m, n) in GG.TRSM_SHAPES:
        for side in "LR":
            for uplo in "UL":
                for ta in "NT":
                    for diag in "UN":
                        for alpha in GG.TRSM_ALPHA:
                            na = m if side == "L" else n
                            A = W.trsm_lower(3000 + idx, na)
                            if uplo == "U":
                                A = np.asfortranarray(A.T)
                            B = W.uniform(4000 + idx, (m, n))
                            F.dtrsm(side, uplo, ta, diag, m, n, alpha, A, na, B, m)
                            ref = golden[f"dtrsm_{idx}"]
                            scale = max(1.0, np.abs(ref).max())
                            assert np.max(np.abs(B - ref)) <= 64 * na * EPS * scale, (
                                idx, side, uplo, ta, diag, alpha)
                            idx += 1


@pytest.mark.parametrize("side,uplo,ta,diag", [
    (s, u, t, d) for s in "LR" for u in "UL" for t in "NT" for d in "UN"])
def test_dtrsm_blocked_vs_oracle(orc, F, gb_clean, side, uplo, ta, diag):
    """Sizes that cross several 32-wide diagonal blocks (GEMM updates active)."""
    m, n = 203, 150
    na = m if side == "L" else n
    A = W.trsm_lower(31, na)
    if uplo == "U":
        A = np.asfortranarray(A.T)
    if diag == "U":
        # unit-diagonal solves of a random triangle grow quickly; keep it tame
        A = np.asfortranarray(np.where(np.eye(na) == 1, A, A / na))
    B = W.uniform(32, (m, n))
    Bo = B.copy(order="F")
    F.dtrsm(side, uplo, ta, diag, m, n, 0.7, A, na, B, m)
    orc.dtrsm(side, uplo, ta, diag, m, n, 0.7, A, na, Bo, m)
    assert np.max(np.abs(B - Bo)) <= 1e3 * na * EPS * max(1.0, np.abs(Bo).max())


def test_dtrsm_config_8192_rows_property(F, gb_clean):
    """Left/Lower/NoTrans/NonUnit with diag n+U(0,1) (the level-3 sweep's TRSM
    operand) on a tall problem: the residual L*X - alpha*B is at rounding level."""
    m, n = 2048, 64
    L = W.trsm_lower(55, m)
    B = W.uniform(56, (m, n))
    X = B.copy(order="F")
    F.dtrsm("L", "L", "N", "N", m, n, 1.0, L, m, X, m)
    res = np.abs(L @ X - B).max() / (np.abs(L).sum(axis=1).max() * np.abs(X).max())
    assert res <= 4 * m * EPS


@pytest.fixture
def emulated_mode(gblib, gb_clean):
    gblib.gb_set_dgemm_mode(1)
    try:
        yield gblib
    finally:
        gblib.gb_set_dgemm_mode(0)


@pytest.mark.parametrize("side,uplo,ta,diag", [
    (s, u, t, d) for s in "LR" for u in "UL" for t in "NT" for d in "UN"])
def test_dtrsm_emulated_recursive_vs_oracle(orc, F, emulated_mode, side, uplo, ta, diag):
    """Emulated-FP64 DTRSM: triangles wider than the 128-wide native leaves
    recurse, the off-diagonal blocks applied by the emulated DGEMM (automatic
    per-tile choice); alpha != 1 and a padded ldb.  Same bound as the native
    blocked solve."""
    m, n = (1100, 300) if side == "L" else (300, 1100)
    na = m if side == "L" else n
    A = W.trsm_lower(71, na)
    if uplo == "U":
        A = np.asfortranarray(A.T)
    if diag == "U":
        A = np.asfortranarray(np.where(np.eye(na) == 1, A, A / na))
    B = np.asfortranarray(W.uniform(72, (m + 5, n)))
    Bo = B.copy(order="F")
    F.dtrsm(side, uplo, ta, diag, m, n, -0.6, A, na, B, m + 5)
    orc.dtrsm(side, uplo, ta, diag, m, n, -0.6, A, na, Bo, m + 5)
    assert np.max(np.abs(B[:m] - Bo[:m])) <= 1e3 * na * EPS * max(1.0, np.abs(Bo[:m]).max())
    assert np.array_equal(B[m:], Bo[m:])


@pytest.mark.parametrize("side,ta", [(s, t) for s in "LR" for t in "NT"])
def test_dtrsm_emulated_leaf_many_vectors(orc, F, emulated_mode, side, ta):
    """The fused FP64 leaves of the emulated DTRSM with many vectors: a 200-wide
    upper triangle (leaves of 128 and 72, forward and backward working orders
    as side and trans vary) against 5000 vectors, the last CTA's 8 lanes idle;
    padded lda and ldb."""
    na, nv = 200, 5000
    m, n = (na, nv) if side == "L" else (nv, na)
    A = np.asfortranarray(np.zeros((na + 3, na)))
    A[:na] = W.trsm_lower(73, na).T
    B = np.asfortranarray(W.uniform(74, (m + 2, n)))
    Bo = B.copy(order="F")
    F.dtrsm(side, "U", ta, "N", m, n, 1.5, A, na + 3, B, m + 2)
    orc.dtrsm(side, "U", ta, "N", m, n, 1.5, A, na + 3, Bo, m + 2)
    assert np.max(np.abs(B[:m] - Bo[:m])) <= 1e3 * na * EPS * max(1.0, np.abs(Bo[:m]).max())
    assert np.array_equal(B[m:], Bo[m:])


def test_dtrsm_emulated_residual(F, emulated_mode):
    """Left/Lower/NoTrans/NonUnit, 2048 x 256 with an exponent-spread right-hand
    side (columns scaled by 2^-40 .. 2^40): L X - B at rounding level column by
    column, i.e. the automatic choice keeps each column's relative accuracy."""
    m, n = 2048, 256
    L = W.trsm_lower(57, m)
    B = W.uniform(58, (m, n)) * np.exp2(np.linspace(-40, 40, n))[None, :]
    X = np.asfortranarray(B.copy())
    F.dtrsm("L", "L", "N", "N", m, n, 1.0, L, m, X, m)
    res = np.abs(L @ X - B).max(axis=0) / (np.abs(L).sum(axis=1).max() * np.abs(X).max(axis=0))
    assert res.max() <= 4 * m * EPS


def test_dsyrk_emulated(orc, F, emulated_mode):
    """Emulated-FP64 DSYRK: the stored triangle within the DMMCH bound, the
    other triangle untouched."""
    n, k = 700, 333
    for uplo in "UL":
        for tr in "NT":
            ra, ca = (n, k) if tr == "N" else (k, n)
            A = W.uniform(62, (ra, ca))
            Cm = W.uniform(63, (n, n))
            C0, Co = Cm.copy(order="F"), Cm.copy(order="F")
            F.dsyrk(uplo, tr, n, k, -1.0, A, ra, 0.5, Cm, n)
            orc.dsyrk(uplo, tr, n, k, -1.0, A, ra, 0.5, Co, n)
            Aop = A if tr == "N" else A.T
            G = np.abs(Aop) @ np.abs(Aop.T) + 0.5 * np.abs(C0)
            tri = np.tril if uplo == "L" else np.triu
            assert dmmch_ratio(tri(Cm), tri(Co), tri(G), k) <= 2 * (k + 2)
            other = np.triu(C0, 1) if uplo == "L" else np.tril(C0, -1)
            got_other = np.triu(Cm, 1) if uplo == "L" else np.tril(Cm, -1)
            assert np.array_equal(other, got_other)


def test_dsyrk_golden_cases(golden, F, gb_clean):
    idx = 0
    for (n, k) in GG.SYRK_SHAPES:
        for uplo in "UL":
            for tr in "NT":
                for (alpha, beta) in GG.SYRK_AB:
                    ra, ca = (n, k) if tr == "N" else (k, n)
                    A = W.uniform(5000 + idx, (ra, ca))
                    Cm = W.uniform(6000 + idx, (n, n))
                    C0 = Cm.copy(order="F")
                    F.dsyrk(uplo, tr, n, k, alpha, A, ra, beta, Cm, n)
                    ref = golden[f"dsyrk_{idx}"]
                    assert np.max(np.abs(Cm - ref)) <= 4 * (k + 2) * EPS * 3, idx
                    other = np.triu(C0, 1) if uplo == "L" else np.tril(C0, -1)
                    got_other = np.triu(Cm, 1) if uplo == "L" else np.tril(Cm, -1)
                    assert np.array_equal(other, got_other), idx
                    idx += 1


def test_dsyrk_large(orc, F, gb_clean):
    n, k = 700, 333
    for uplo in "UL":
        for tr in "NT":
            ra, ca = (n, k) if tr == "N" else (k, n)
            A = W.uniform(60, (ra, ca))
            Cm = W.uniform(61, (n, n))
            Co = Cm.copy(order="F")
            F.dsyrk(uplo, tr, n, k, -1.0, A, ra, 0.5, Cm, n)
            orc.dsyrk(uplo, tr, n, k, -1.0, A, ra, 0.5, Co, n)
            assert np.max(np.abs(Cm - Co)) <= 4 * (k + 2) * EPS * k


def test_dgemm_batch_grouped(orc, gb_clean):
    ns = gb.cblas()
    import ctypes as C
    groups = [(17, 9, 33, "N", "T", 1.0, 0.0, 3), (40, 41, 8, "T", "N", -0.5, 2.0, 2)]
    ta, tb, ms, ns_, ks, al, be, lda, ldb, ldc, gs = ([] for _ in range(11))
    Aps, Bps, Cps, keep, refs = [], [], [], [], []
    seed = 900
    for (m, n, k, a, b, alpha, beta, cnt) in groups:
        ta.append(abi.CblasNoTrans if a == "N" else abi.CblasTrans)
        tb.append(abi.CblasNoTrans if b == "N" else abi.CblasTrans)
        ms.append(m); ns_.append(n); ks.append(k); al.append(alpha); be.append(beta)
        gs.append(cnt)
        for _ in range(cnt):
            A, B, Cm = W.gemm_operands(seed, m, n, k, a, b, pad=1)
            seed += 3
            Co = Cm.copy(order="F")
            orc.dgemm(a, b, m, n, k, alpha, A, A.shape[0], B, B.shape[0], beta, Co, Co.shape[0])
            keep += [A, B, Cm]
            refs.append((Cm, Co, k))
            Aps.append(A.ctypes.data); Bps.append(B.ctypes.data); Cps.append(Cm.ctypes.data)
        lda.append(A.shape[0]); ldb.append(B.shape[0]); ldc.append(Cm.shape[0])

    def iarr(v):
        return (C.c_int * len(v))(*v)

    ns.cblas_dgemm_batch(abi.CblasColMajor, iarr(ta), iarr(tb), iarr(ms), iarr(ns_), iarr(ks),
                         (C.c_double * 2)(*al), (C.c_void_p * len(Aps))(*Aps), iarr(lda),
                         (C.c_void_p * len(Bps))(*Bps), iarr(ldb), (C.c_double * 2)(*be),
                         (C.c_void_p * len(Cps))(*Cps), iarr(ldc), 2, iarr(gs))
    for (Cm, Co, k) in refs:
        assert np.max(np.abs(Cm - Co)) <= 4 * (k + 2) * EPS * k * 4
