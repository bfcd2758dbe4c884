"""Pins the oracle (C restatement of the reference algorithms) against golden
vectors produced by an OpenBLAS build (tests/golden/gen_golden.py)."""
from __future__ import annotations

import sys
import os

import numpy as np
import pytest

from conftest import EPS, dmmch_ratio

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import gen_golden as GG  # noqa: E402

from openblas_gb300 import workloads as W  # noqa: E402


def test_prng_known_answer():
    # splitmix64 with seed 0: the first outputs of the published generator
    z = W.splitmix64(0, 2)
    assert int(z[0]) == 0xE220A8397B1DCDAF
    assert int(z[1]) == 0x6E789E6AA1B965F4


def test_golden_provenance(golden):
    assert "OpenBLAS" in str(golden["openblas_config"])


def test_dgemm_cases(golden, orc):
    idx = 0
    for (m, n, k) in GG.GEMM_SHAPES:
        for (alpha, beta) in GG.GEMM_AB:
            for ta in "NT":
                for tb in "NT":
                    A, B, Cm = W.gemm_operands(GG.gemm_case_seed(idx), m, n, k, ta, tb, pad=3)
                    C0 = Cm.copy(order="F")
                    if beta == 0.0:
                        Cm[:m, :n] = np.nan
                    orc.dgemm(ta, tb, m, n, k, alpha, A, A.shape[0], B, B.shape[0], beta, Cm,
                              Cm.shape[0])
                    ref = golden[f"dgemm_{idx}"]
                    assert not np.isnan(Cm[:m, :n]).any()
                    G = orc.dgemm_absbound(ta, tb, m, n, k, alpha, A, A.shape[0], B, B.shape[0],
                                           0.0 if beta == 0 else beta, C0, C0.shape[0])
                    assert dmmch_ratio(Cm[:m, :n], ref, G, k) <= 2 * (k + 2), (idx, m, n, k)
                    # padding rows untouched
                    assert np.array_equal(Cm[m:, :], C0[m:, :])
                    idx += 1


def test_double_double_gemm_against_exact_sums(orc):
    """The double-double GEMM is the accuracy yardstick of the emulated FP64
    engine, so it is pinned itself: against exact rational sums of
    alpha*A*B + beta*C.  Two cases:
    - operands spread over 2^±20;
    - columns of B built to cancel almost all of each dot product (with and
      without a beta*C term).
    The result must be the exact value rounded to double, up to a
    double-double residue: |dd - exact| <= 2^-53 |exact| + 2^-100 G."""
    from fractions import Fraction

    m, n, k = 6, 5, 240
    cases = []
    A = np.asfortranarray(W.exponent_spread(300, (m, k), 20))
    B = np.asfortranarray(W.exponent_spread(301, (k, n), 20))
    cases.append((A, B, 1.0, 0.0))
    # cancellation: A's second half repeats its first and B's second half negates its
    # first, so every dot product is one small perturbed term
    A2 = np.asfortranarray(W.uniform(302, (m, k)))
    B2 = np.asfortranarray(W.uniform(303, (k, n)))
    h = k // 2
    A2[:, h:] = A2[:, :h]
    B2[h:, :] = -B2[:h, :]
    B2[0, :] += 2.0 ** -40
    cases.append((A2, B2, -1.5, 0.75))
    cases.append((A2, B2, -1.5, 0.0))  # the cancelled dot product alone
    for A, B, alpha, beta in cases:
        C0 = np.asfortranarray(W.uniform(304, (m, n)))
        C = C0.copy(order="F")
        orc.dgemm_dd("N", "N", m, n, k, alpha, A, m, B, k, beta, C, m)
        for i in range(m):
            for j in range(n):
                dot = sum(Fraction(float(A[i, p])) * Fraction(float(B[p, j])) for p in range(k))
                exact = Fraction(alpha) * dot + Fraction(beta) * Fraction(float(C0[i, j]))
                G = abs(alpha) * float(np.abs(A[i]) @ np.abs(B[:, j])) + abs(beta * C0[i, j])
                err = abs(Fraction(float(C[i, j])) - exact)
                assert err <= Fraction(2.0 ** -53) * abs(exact) + Fraction(2.0 ** -100) * \
                    Fraction(G), (i, j, float(err), float(exact))


def test_dgemm_c1(golden, orc):
    A, B, Cm = W.gemm_operands(42, 1024, 1024, 1024)
    orc.dgemm("N", "N", 1024, 1024, 1024, 1.5, A, 1024, B, 1024, 0.5, Cm, 1024)
    assert np.allclose(Cm.sum(axis=0), golden["dgemm_c1_colsum"], rtol=0, atol=1e-9)
    assert np.max(np.abs(Cm[::37, ::41] - golden["dgemm_c1_sample"])) < 1e-11


def test_dtrsm_cases(golden, orc):
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
                            orc.dtrsm(side, uplo, ta, diag, m, n, alpha, A, na, B, m)
                            ref = golden[f"dtrsm_{idx}"]
                            scale = max(1.0, np.abs(ref).max())
                            assert np.max(np.abs(B - ref)) <= 64 * na * EPS * scale, idx
                            idx += 1


def test_dsyrk_cases(golden, orc):
    idx = 0
    for (n, k) in GG.SYRK_SHAPES:
        for uplo in "UL":
            for tr in "NT":
                for (alpha, beta) in GG.SYRK_AB:
                    ra, ca = (n, k) if tr == "N" else (k, n)
                    A = W.uniform(5000 + idx, (ra, ca))
                    Cm = W.uniform(6000 + idx, (n, n))
                    orc.dsyrk(uplo, tr, n, k, alpha, A, ra, beta, Cm, n)
                    ref = golden[f"dsyrk_{idx}"]
                    assert np.max(np.abs(Cm - ref)) <= 4 * (k + 2) * EPS * 3, idx
                    idx += 1


def test_dgetrf_cases(golden, orc):
    for idx, (m, n) in enumerate(GG.GETRF_SHAPES):
        A = W.uniform(7000 + idx, (m, n))
        ipiv = np.zeros(min(m, n), np.int32)
        info = orc.dgetrf(m, n, A, m, ipiv)
        assert info == int(golden[f"dgetrf_{idx}_info"])
        assert np.array_equal(ipiv, golden[f"dgetrf_{idx}_ipiv"]), (m, n)
        if f"dgetrf_{idx}_lu" in golden:
            assert np.max(np.abs(A - golden[f"dgetrf_{idx}_lu"])) < 1e-11
    for n in GG.GETRF_PIV_ONLY:
        A = W.uniform(7100 + n, (n, n))
        ipiv = np.zeros(n, np.int32)
        assert orc.dgetrf(n, n, A, n, ipiv) == int(golden[f"dgetrf_piv{n}_info"])
        assert np.array_equal(ipiv, golden[f"dgetrf_piv{n}"])


def test_dgetrf_singular(golden, orc):
    A = W.uniform(7200, (9, 9))
    A[:, 3] = 0.0
    ipiv = np.zeros(9, np.int32)
    assert orc.dgetrf(9, 9, A, 9, ipiv) == int(golden["dgetrf_sing_info"]) == 4
    assert np.array_equal(ipiv, golden["dgetrf_sing_ipiv"])
    assert np.max(np.abs(A - golden["dgetrf_sing_lu"])) < 1e-12


def test_dgetrs_dgesv(golden, orc):
    for t, trans in enumerate("NT"):
        for nrhs in (1, 5):
            n = 64
            A = W.uniform(7300 + t, (n, n))
            ipiv = np.zeros(n, np.int32)
            orc.dgetrf(n, n, A, n, ipiv)
            B = W.uniform(7400 + nrhs, (n, nrhs))
            orc.dgetrs(trans, n, nrhs, A, n, ipiv, B, n)
            ref = golden[f"dgetrs_{trans}_{nrhs}"]
            assert np.max(np.abs(B - ref)) <= 1e-10 * max(1, np.abs(ref).max())
    A = W.uniform(7500, (100, 100))
    B = W.uniform(7501, (100, 3))
    ipiv = np.zeros(100, np.int32)
    assert orc.dgesv(100, 3, A, 100, ipiv, B, 100) == int(golden["dgesv_info"])
    assert np.array_equal(ipiv, golden["dgesv_ipiv"])
    assert np.max(np.abs(B - golden["dgesv_x"])) <= 1e-10 * np.abs(B).max()


def test_dpotrf_cases(golden, orc):
    for n in GG.POTRF_N:
        for uplo in "LU":
            A = W.spd(8000 + n, n)
            assert orc.dpotrf(uplo, n, A, n) == int(golden[f"dpotrf_{uplo}_{n}_info"]) == 0
            ref = golden[f"dpotrf_{uplo}_{n}"]
            tri = np.tril if uplo == "L" else np.triu
            assert np.max(np.abs(tri(A) - tri(ref))) < 1e-12
            # the other triangle is not referenced
            other = np.triu if uplo == "L" else np.tril
            assert np.array_equal(other(A, 1 if uplo == "L" else -1),
                                  other(W.spd(8000 + n, n), 1 if uplo == "L" else -1))
    A = W.spd(8100, 20)
    A[11, 11] = -1.0
    info = orc.dpotrf("L", 20, A, 20)
    assert info == int(golden["dpotrf_npd_info"]) == 12
    ref = golden["dpotrf_npd"]
    assert np.max(np.abs(np.tril(A)[:, :12] - np.tril(ref)[:, :12])) < 1e-12


def test_dlaswp_cases(golden, orc):
    for idx, (n, k1, k2, incx) in enumerate(GG.LASWP_CASES):
        rows = 12
        A = W.uniform(8200 + idx, (rows, n))
        ipiv = golden[f"dlaswp_{idx}_ipiv"].astype(np.int32)
        orc.dlaswp(n, A, rows, k1, k2, ipiv, incx)
        assert np.array_equal(A, golden[f"dlaswp_{idx}"]), (n, k1, k2, incx)


def test_dsgesv_cases(golden, orc):
    for idx, (n, nrhs) in enumerate(GG.DSGESV_CASES):
        A = W.uniform(8400 + idx, (n, n))
        B = W.uniform(8500 + idx, (n, nrhs))
        X = np.zeros((n, nrhs), order="F")
        ipiv = np.zeros(n, np.int32)
        info, it = orc.dsgesv(n, nrhs, A, n, ipiv, B, n, X, n)
        assert info == int(golden[f"dsgesv_{idx}_info"]) == 0
        assert it == int(golden[f"dsgesv_{idx}_iter"])
        assert np.array_equal(ipiv, golden[f"dsgesv_{idx}_ipiv"])
        assert np.max(np.abs(X - golden[f"dsgesv_{idx}_x"])) <= 64 * n * EPS * np.abs(X).max()
    n = 60
    A = W.ill_conditioned(8600, n, 12)
    B = W.uniform(8601, (n, 1))
    X = np.zeros((n, 1), order="F")
    ipiv = np.zeros(n, np.int32)
    info, it = orc.dsgesv(n, 1, A, n, ipiv, B, n, X, n)
    assert it == int(golden["dsgesv_ill_iter"]) and it < 0
    assert np.array_equal(ipiv, golden["dsgesv_ill_ipiv"])
    # kappa = 1e12: forward errors are ~kappa*eps, so compare backward errors
    A = W.ill_conditioned(8600, n, 12)
    for Xs in (X, golden["dsgesv_ill_x"]):
        r = B - A @ Xs
        berr = np.abs(r).max() / (np.abs(A).sum(axis=1).max() * np.abs(Xs).max() + np.abs(B).max())
        assert berr <= n * EPS
    assert np.max(np.abs(X - golden["dsgesv_ill_x"])) <= 1e-3 * np.abs(X).max()


def test_sgetrf_pivots(golden, orc):
    for n in (128, 256):
        A = W.uniform(8700 + n, (n, n)).astype(np.float32)
        A = np.asfortranarray(A)
        ipiv = np.zeros(n, np.int32)
        assert orc.sgetrf(n, n, A, n, ipiv) == int(golden[f"sgetrf_{n}_info"])
        assert np.array_equal(ipiv, golden[f"sgetrf_{n}_ipiv"])
        if f"sgetrf_{n}_lu" in golden:
            assert np.max(np.abs(A - golden[f"sgetrf_{n}_lu"])) < 1e-3


def test_dpotrs_cases(golden, orc):
    for idx, (uplo, n, nrhs) in enumerate(GG.DPOTRS_CASES):
        A = W.spd(8800 + idx, n)
        assert orc.dpotrf(uplo, n, A, n) == 0
        B = W.uniform(8810 + idx, (n, nrhs))
        assert orc.dpotrs(uplo, n, nrhs, A, n, B, n) == int(golden[f"dpotrs_{idx}_info"]) == 0
        ref = golden[f"dpotrs_{idx}_x"]
        assert np.max(np.abs(B - ref)) <= 64 * n * EPS * np.abs(ref).max()


def test_dsposv_cases(golden, orc):
    for idx, (uplo, n, nrhs) in enumerate(GG.DSPOSV_CASES):
        A = W.spd(8900 + idx, n)
        B = W.uniform(8910 + idx, (n, nrhs))
        X = np.zeros((n, nrhs), order="F")
        info, it = orc.dsposv(uplo, n, nrhs, A, n, B, n, X, n)
        assert info == int(golden[f"dsposv_{idx}_info"]) == 0
        assert it == int(golden[f"dsposv_{idx}_iter"])
        ref = golden[f"dsposv_{idx}_x"]
        assert np.max(np.abs(X - ref)) <= 64 * n * EPS * np.abs(ref).max()


def test_dsposv_fallbacks(golden, orc):
    n = 60
    A = W.spd_ill_conditioned(8920, n, 10)
    B = W.uniform(8921, (n, 1))
    X = np.zeros((n, 1), order="F")
    info, it = orc.dsposv("L", n, 1, A.copy(order="F"), n, B, n, X, n)
    assert info == int(golden["dsposv_ill_info"]) == 0
    assert it == int(golden["dsposv_ill_iter"]) and it < 0
    A = W.spd(8930, 30)
    A[17, 17] = -1.0
    B = W.uniform(8931, (30, 1))
    X = np.zeros((30, 1), order="F")
    info, it = orc.dsposv("L", 30, 1, A, 30, B, 30, X, 30)
    assert info == int(golden["dsposv_npd_info"]) == 18
    assert it == int(golden["dsposv_npd_iter"]) == -3


def _tri_other(uplo, X):
    return np.triu(X, 1) if uplo == "L" else np.tril(X, -1)


def test_dtrmm_cases(golden, orc):
    idx = 0
    for (m, n) in GG.TRSM_SHAPES:
        for side in "LR":
            for uplo in "UL":
                for ta in "NT":
                    for diag in "UN":
                        for alpha in GG.TRSM_ALPHA:
                            A, B = GG.trmm_operands(idx, side, uplo, m, n)
                            orc.dtrmm(side, uplo, ta, diag, m, n, alpha, A, A.shape[0], B, m)
                            ref = golden[f"dtrmm_{idx}"]
                            scale = max(1.0, np.abs(ref).max())
                            assert np.max(np.abs(B - ref)) <= 4 * A.shape[0] * EPS * scale, idx
                            idx += 1


def test_dsyr2k_cases(golden, orc):
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
                    orc.dsyr2k(uplo, tr, n, k, alpha, A, ra, B, ra, beta, Cm, n)
                    ref = golden[f"dsyr2k_{idx}"]
                    assert np.max(np.abs(Cm - ref)) <= 8 * (k + 2) * EPS * max(1, np.abs(ref).max())
                    assert np.array_equal(_tri_other(uplo, Cm), _tri_other(uplo, C0))
                    idx += 1


def test_dgemmt_cases(golden, orc):
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
                        orc.dgemmt(uplo, ta, tb, m, k, alpha, A, A.shape[0], B, B.shape[0],
                                   beta, Cm, m)
                        ref = golden[f"dgemmt_{idx}"]
                        assert np.max(np.abs(Cm - ref)) <= 4 * (k + 2) * EPS * max(1, np.abs(ref).max())
                        assert np.array_equal(_tri_other(uplo, Cm), _tri_other(uplo, C0))
                        idx += 1


@pytest.mark.parametrize("name,dt", GG.ZGEMM_ROUTINES)
def test_complex_gemm_cases(golden, orc, name, dt):
    """ZGEMM/CGEMM (componentwise bound) and the 3M forms (normwise bound)
    for every op pair N/T/R/C, alpha/beta edge values and beta = 0 over NaN."""
    from conftest import zgemm_ratio
    eps = float(np.finfo(np.float32 if dt == np.complex64 else np.float64).eps)
    for idx, (m, n, k, ta, tb, al, be) in enumerate(GG.zgemm_cases()):
        A, B, Cm = GG.complex_operands(idx, m, n, k, ta, tb, dt)
        C0 = Cm.copy(order="F")
        if be == 0:
            Cm[:m, :n] = np.nan
        getattr(orc, name)(ta, tb, m, n, k, al, A, A.shape[0], B, B.shape[0], be, Cm,
                           Cm.shape[0])
        ref = golden[f"{name}_{idx}"]
        r = zgemm_ratio(Cm, ref, A, B, C0, m, n, k, ta, tb, al, be, eps,
                        normwise=name.endswith("3m"))
        assert r <= 4 * (k + 2), (name, idx, m, n, k, ta, tb, r)
        assert np.array_equal(Cm[m:], C0[m:])  # padding rows untouched
