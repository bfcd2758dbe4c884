"""The emulated-FP64 DGEMM scheme, checked on the CPU.

A model of the device pipeline in exact integer arithmetic: per-row (op(A))
and per-column (op(B)) exponents e = frexp exponent of the largest |x|, the
value truncated toward zero to 8*S bits below 2^e and cut into S signed
8-bit digits, level sums P_L = sum_{s+t=L} A_s B_t^T for L = 2..S+1 (the
triangle of S(S+1)/2 products), and one rounding of sum_L P_L 2^(8(S+1-L))
to FP64 before the exact scale alpha * 2^(e_i + f_j - 8(S+1)).  The device
rounds that sum with a sticky bit and a round-to-nearest conversion, which
is the correctly rounded value that Python's int -> float conversion gives.
For one K segment, beta = 0, finite operands and results that are normal
numbers, the model is the device's arithmetic step by step.

The tests check the digit decomposition, the exactness bounds the device
relies on (read from the kernel source, so the constants cannot drift), and
the accuracy the scheme delivers against the double-double oracle -- the
same bounds that the GPU parity tests apply to the device result.
"""
from __future__ import annotations

import os
import re

import numpy as np
import pytest

from conftest import EPS

from openblas_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIGIT_BITS = 8


def exponents(X: np.ndarray, axis: int) -> np.ndarray:
    """frexp exponent of max |x| along ``axis`` (0 for an all-zero line):
    |x| < 2^e on the line."""
    mx = np.abs(X).max(axis=axis)
    _, e = np.frexp(mx)
    return np.where(mx == 0, 0, e).astype(np.int64)


def digits(X: np.ndarray, e_line: np.ndarray, axis: int, S: int) -> np.ndarray:
    """Signed digits, shape (S, *X.shape): X ~= 2^e * sum_s d_s 2^(-8s),
    truncated toward zero."""
    e = np.expand_dims(e_line, axis)
    m, ex = np.frexp(np.abs(X))                    # |x| = m 2^ex, m in [0.5, 1)
    M = (m * 2.0 ** 53).astype(np.uint64)          # exact 53-bit integer mantissa
    sh = ex.astype(np.int64) - 53 + DIGIT_BITS * S - e
    left = np.where(sh > 0, sh, 0).astype(np.uint64)
    right = np.where(sh < 0, np.minimum(-sh, 63), 0).astype(np.uint64)
    t = np.where(sh >= 0, M << left, M >> right)
    t = np.where((X == 0) | (sh <= -64), np.uint64(0), t)
    sign = np.where(np.signbit(X), -1, 1).astype(np.int64)
    out = np.empty((S,) + X.shape, np.int64)
    for s in range(1, S + 1):
        d = (t >> np.uint64(DIGIT_BITS * (S - s))) & np.uint64((1 << DIGIT_BITS) - 1)
        out[s - 1] = sign * d.astype(np.int64)
    return out


def level_sums(Ad: np.ndarray, Bd: np.ndarray, S: int) -> list[np.ndarray]:
    """P_L for L = 2..S+1 as exact int64.  Digit products summed over k stay
    below k * 255^2 * S < 2^53, so the FP64 matrix product is exact."""
    k = Ad.shape[2]
    assert k * 255 * 255 * S < 2 ** 53
    P = []
    for L in range(2, S + 2):
        acc = np.zeros((Ad.shape[1], Bd.shape[2]))
        for s in range(1, L):
            acc += Ad[s - 1].astype(np.float64) @ Bd[L - s - 1].astype(np.float64)
        P.append(acc.astype(np.int64))
    return P


def emulated_gemm(A: np.ndarray, B: np.ndarray, S: int, alpha: float = 1.0) -> np.ndarray:
    """alpha * A @ B by the slice scheme (beta = 0, one K segment)."""
    ea, fb = exponents(A, 1), exponents(B, 0)
    P = level_sums(digits(A, ea, 1, S), digits(B, fb, 0, S), S)
    acc = np.zeros(P[0].shape, dtype=object)
    for L, PL in zip(range(2, S + 2), P):
        acc = acc + PL.astype(object) * (1 << (DIGIT_BITS * (S + 1 - L)))
    t = acc.astype(np.float64)                     # one correctly rounded conversion
    x = ea[:, None] + fb[None, :] - DIGIT_BITS * (S + 1)
    # t * alpha rounded once, then the power of two.  Where alpha * 2^x is a
    # normal number the device multiplies by it instead, which gives the same
    # value whenever the result is a normal number.
    m_alpha, e_alpha = np.frexp(alpha)
    return np.ldexp(t * m_alpha, x + e_alpha)


def _dd(orc, A, B, alpha=1.0):
    m, k = A.shape
    n = B.shape[1]
    A, B = np.asfortranarray(A), np.asfortranarray(B)
    C = np.zeros((m, n), order="F")
    orc.dgemm_dd("N", "N", m, n, k, alpha, A, m, B, k, 0.0, C, m)
    return C


# ------------------------------------------------------------------ constants
def _const(src: str, name: str) -> int:
    m = re.search(r"constexpr int[^;]*\b" + name + r"\s*=\s*(\d+)", src)
    assert m, name
    return int(m.group(1))


def _csrc(*names):
    return "".join(open(os.path.join(ROOT, "openblas_gb300", "csrc", n)).read() for n in names)


def test_exactness_bounds_of_the_kernel_constants():
    src = _csrc("ozaki_digits.cuh", "ozaki.cu", "gb_internal.h")
    bits = _const(src, "DIGIT_BITS")
    bk = _const(src, "BK")
    chunk = bk * _const(src, "KC_BLOCKS")            # FP32 accumulation depth in TMEM
    seg = int(re.search(r"EMU_K_SEGMENT\s*=\s*(\d+)", src).group(1))  # int32 level-sum depth
    dmax = (1 << bits) - 1
    assert bits == DIGIT_BITS
    assert chunk * dmax * dmax < 2 ** 24             # every FP32 partial sum is an exact integer
    max_slices = 8
    assert max_slices * seg * dmax * dmax < 2 ** 31  # a level sum of up to 8 products fits int32
    assert bits * max_slices <= 64                   # the truncated value fits 64 bits
    # sum_L |P_L| 2^(8(S+1-L)) < 2^127: the int128 recombine cannot overflow
    worst = sum((L - 1) * seg * dmax * dmax * 2 ** (bits * (max_slices + 1 - L))
                for L in range(2, max_slices + 2))
    assert worst < 2 ** 127


# ------------------------------------------------------------------ digits
@pytest.mark.parametrize("S", [3, 6, 7, 8])
def test_digits_reconstruct_the_truncated_value(S):
    X = W.exponent_spread(5, (40, 300), 30)
    X[3] = 0.0
    X[7, 5] = 5e-310                                  # subnormal next to normal values
    X[11, :] = 2.0 ** -1060                           # a wholly subnormal row
    X[12, 9] = -1.0
    e = exponents(X, 1)
    d = digits(X, e, 1, S)
    assert np.abs(d).max() <= 255
    recon = np.zeros(X.shape, dtype=object)
    for s in range(1, S + 1):
        recon = recon + d[s - 1].astype(object) * (1 << (DIGIT_BITS * (S - s)))
    # recon = trunc(x * 2^(8S - e)) exactly (rational arithmetic), so the
    # truncation error is below one unit of the last digit, 2^(e - 8S)
    for i in range(X.shape[0]):
        sh = DIGIT_BITS * S - int(e[i])
        for j in range(X.shape[1]):
            x = float(X[i, j])
            r = int(recon[i, j])
            num, den = abs(x).as_integer_ratio()
            tr = (num << sh) // den if sh >= 0 else num // (den << -sh)
            assert abs(r) == tr and (r <= 0 if x < 0 else r >= 0), (i, j, x, r, tr)


# ------------------------------------------------------------------ products
def test_integer_operands_exact():
    A = W.randint(1, (40, 600), -127, 127).astype(np.float64)
    B = W.randint(2, (600, 30), -127, 127).astype(np.float64)
    C = emulated_gemm(A, B, 7)
    assert np.array_equal(C, (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64))


def test_worst_case_digits_exact():
    k = 4096
    A = np.full((6, k), 255.0)
    A[::2] = -255.0
    B = np.full((k, 5), 255.0)
    C = emulated_gemm(A, B, 7)
    exact = np.where(np.arange(6)[:, None] % 2 == 0, -1.0, 1.0) * (k * 255.0 * 255.0)
    assert np.array_equal(C, np.broadcast_to(exact, C.shape))


def test_elementwise_error_bound(orc):
    """|C - C_exact| <= |alpha| k (S+4) 2^(e_i+f_j-8S) + 2 eps |C_exact|: truncation of
    both operands (2 units of 2^-8S per product) plus the dropped levels s+t > S+1
    (at most (S+1) 2^-8S per product), and one final rounding."""
    S, alpha = 7, -1.75
    A = W.exponent_spread(40, (64, 500), 12)
    B = W.exponent_spread(41, (500, 48), 12)
    C = emulated_gemm(A, B, S, alpha)
    Cx = _dd(orc, A, B, alpha)
    ea, fb = exponents(A, 1), exponents(B, 0)
    k = A.shape[1]
    bound = (abs(alpha) * k * (S + 4) * np.ldexp(1.0, ea[:, None] + fb[None, :] - 8 * S)
             + 2 * EPS * np.abs(Cx))
    assert np.all(np.abs(C - Cx) <= bound)


@pytest.mark.parametrize("alpha", [1.0, -1.5])
def test_results_near_the_underflow_threshold(alpha):
    """Rows of A near 2^-512 and columns of B near 2^-500 give C near 2^-1010,
    still normal numbers.  The recombine's power-of-two scale alone
    (alpha * 2^(e_i + f_j - 8(S+1))) is far below the smallest subnormal
    there, so the scaling must not form it on its own; the results must be
    the exactly rounded products up to the usual 56-bit truncation."""
    from fractions import Fraction

    A = W.uniform(70, (5, 40)) * 2.0 ** -512
    B = W.uniform(71, (40, 4)) * 2.0 ** -500
    C = emulated_gemm(A, B, 7, alpha)
    for i in range(5):
        for j in range(4):
            exact = Fraction(alpha) * sum(Fraction(float(A[i, p])) * Fraction(float(B[p, j]))
                                          for p in range(40))
            G = abs(alpha) * float(np.abs(A[i]) @ np.abs(B[:, j]))
            assert abs(float(exact)) > np.finfo(np.float64).tiny      # a normal result
            assert abs(Fraction(float(C[i, j])) - exact) <= Fraction(8 * EPS) * Fraction(G)


# the (exponent spread, slices, bound) cases the device parity tests use
@pytest.mark.parametrize("e,slices,bound", [(0, 7, 8), (0, 6, 200), (8, 7, 32), (16, 7, 256),
                                            (0, 8, 8)])
def test_normwise_accuracy_vs_double_double(orc, e, slices, bound):
    m = n = k = 192
    A = W.exponent_spread(10 + e, (m, k), e)
    B = W.exponent_spread(20 + e, (k, n), e)
    C = emulated_gemm(A, B, slices)
    Cx = _dd(orc, A, B)
    G = np.abs(A) @ np.abs(B)
    err = np.abs(C - Cx).max() / G.max()
    assert err <= bound * EPS, err / EPS


def test_fewer_slices_lose_accuracy(orc):
    A = W.uniform(60, (64, 256))
    B = W.uniform(61, (256, 64))
    Cx = _dd(orc, A, B)
    G = (np.abs(A) @ np.abs(B)).max()
    errs = [np.abs(emulated_gemm(A, B, S) - Cx).max() / G for S in (3, 4, 5, 6, 7)]
    for lo, hi in zip(errs[1:], errs[:-1]):
        assert lo < hi / 16                          # each slice adds 8 bits
    assert errs[0] > 2 ** -30


def test_exactness_bounds_of_the_batched_emulated_kernel():
    """The grouped emulated DGEMM sums one 64-deep chunk of a digit product in
    FP32 (mma.sync) and the level sums over all chunks of K <= EM_KMAX in
    int32; both must stay exact."""
    src = _csrc("ozaki_digits.cuh", "batched.cu")
    bits = _const(src, "DIGIT_BITS")
    dmax = (1 << bits) - 1
    kc, kmax, s = _const(src, "EM_KC"), _const(src, "EM_KMAX"), _const(src, "EM_S")
    assert kc % 16 == 0                          # whole m16n8k16 steps
    assert kc * dmax * dmax < 2 ** 24            # one chunk of one product is exact in FP32
    assert s * kmax * dmax * dmax < 2 ** 31      # a level sum (<= S products) fits int32
    assert bits * s <= 64
