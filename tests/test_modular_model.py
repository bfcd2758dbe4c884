"""The modular scheme of the emulated DGEMM, restated on the CPU.

The automatic mode of the emulated DGEMM may compute a column tile of C from
residues: op(A) and op(B) are cut to t-bit integers A', B', each residue
product (A' mod p_l)(B' mod p_l) runs on the tensor cores like a digit-slice
product, and the Chinese remainder theorem recovers C' = A'B' exactly.
These tests take the moduli and chunk constants from the CUDA source and
check, in exact integer arithmetic:

* the moduli are odd, pairwise coprime and at most 511, so a symmetric
  residue has |r| <= 255 (exact in bf16, and a 256-deep FP32 chunk of
  residue products stays below 2^24, as for 8-bit digits);
* the bit count t chosen for a K segment keeps every |C'| < k 2^2t below
  M / 2 with room for the rounded CRT quotient (t = 55 for K = 8192);
* the residues the split kernel forms in FP32 from 12-bit chunks and
  symmetric chunk weights equal the exact symmetric residues with no
  correction step (the rounded quotient is exact), over random and extreme
  t-bit integers of both signs;
* the residue GEMM's epilogue reduction (offset, then the quotient from a
  multiply-high by ceil(2^40 / p)) equals the residue for every sum an
  8192-deep segment can produce;
* the reconstruction (moduli combined in pairs with 32-bit arithmetic, the
  quotient from 32-bit fixed-point fractions, four signed 64-bit limbs, the
  value taken modulo 2^128) returns C' for random and extreme values of C',
  including +-(k 2^2t - 1).
"""
from __future__ import annotations

import math
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "openblas_gb300", "csrc")


def _src():
    with open(os.path.join(CSRC, "ozaki.cu")) as f:
        return f.read()


def _const(src, name):
    return int(re.search(r"constexpr int " + name + r"\s*=\s*(\d+)", src).group(1))


SRC = _src()
MODULI = [int(x) for x in
          re.search(r"MODULI\[MOD_COUNT\]\s*=\s*\{([^}]*)\}", SRC).group(1).replace("\n", " ")
          .split(",")]
MOD_COUNT = _const(SRC, "MOD_COUNT")
CHUNK_BITS = _const(SRC, "MOD_CHUNK_BITS")
CHUNKS = _const(SRC, "MOD_CHUNKS")
M = math.prod(MODULI)


def mod_bits(k):
    """The largest t <= 60 with M > 2 k 2^2t (1 + 2^-6) (ozaki.cu mod_bits)."""
    kb = 0
    while kb < 63 and (1 << kb) < k:
        kb += 1
    for t in range(CHUNK_BITS * CHUNKS, 0, -1):
        if 2 * t + 1 + kb > 126:
            continue
        lhs = k << (2 * t + 1)
        if lhs + (lhs >> 6) < M:
            return t
    return 0


def crt_table():
    """The reconstruction's constants: moduli paired (a_i, b_i) = (p_2i,
    p_2i+1), m_i = a_i b_i; a_i^-1 mod b_i, ceil(2^32 / b_i), and the CRT
    weights W_i = (M / m_i) u_i with u_i = (M / m_i)^-1 mod m_i and their
    32-bit fixed-point fractions F_i = round(2^32 u_i / m_i)."""
    pairs = []
    for i in range(0, MOD_COUNT, 2):
        a, b = MODULI[i], MODULI[i + 1]
        mi = a * b
        u = pow((M // mi) % mi, -1, mi)
        F = ((u << 32) // mi) + (1 if ((u << 32) % mi) * 2 >= mi else 0)
        pairs.append(dict(a=a, b=b, inv=pow(a, -1, b), magic=((1 << 32) + b - 1) // b,
                          W=(M // mi) * u, F=F))
    return pairs


def reconstruct(residues, pairs):
    """C' from its residues in [0, p_l), as the reconstruction kernel forms it:
    each pair combined in 32-bit arithmetic, then the CRT over the pairs in
    four signed 64-bit limbs, the value taken modulo 2^128."""
    ys = []
    for i, pr in enumerate(pairs):
        ra, rb, a, b = residues[2 * i], residues[2 * i + 1], pr["a"], pr["b"]
        u = ((rb + 2 * b - ra) * pr["inv"]) & 0xFFFFFFFF
        assert 0 <= u < 1 << 20
        t = u - ((u * pr["magic"]) >> 32) * b
        assert 0 <= t < b
        ys.append(ra + a * t)
    qa = sum(y * pr["F"] for y, pr in zip(ys, pairs))
    assert qa < 1 << 64
    q = (qa + (1 << 31)) >> 32
    limbs = []
    for j in range(4):
        a = sum(y * ((pr["W"] >> (32 * j)) & 0xFFFFFFFF) for y, pr in zip(ys, pairs))
        a -= q * ((M >> (32 * j)) & 0xFFFFFFFF)
        assert abs(a) < (1 << 53)                # a signed 64-bit limb
        limbs.append(a)
    u = sum(a << (32 * j) for j, a in enumerate(limbs)) % (1 << 128)
    return u - (1 << 128) if u >= (1 << 127) else u


def test_moduli_are_odd_coprime_and_small():
    assert len(MODULI) == MOD_COUNT == 14
    for i, p in enumerate(MODULI):
        assert p % 2 == 1 and p <= 511
        for q in MODULI[i + 1:]:
            assert math.gcd(p, q) == 1
    assert 256 * 255 * 255 < 2 ** 24           # a residue-product chunk is exact in FP32
    assert 2 ** 125 < M < 2 ** 126


def test_bit_count_keeps_products_below_half_the_modulus():
    assert mod_bits(4096) == 56 and mod_bits(8192) == 55
    for k in (1, 2, 3, 64, 255, 256, 257, 1000, 4095, 4096, 5000, 65536):
        t = mod_bits(k)
        assert 1 <= t <= CHUNK_BITS * CHUNKS
        bound = k * (1 << (2 * t))              # |C'| < k 2^2t
        assert 2 * bound * (1 + 2 ** -6) < M
        assert bound < (1 << 127)
        if t < CHUNK_BITS * CHUNKS:              # t is the largest such count
            assert 2 * k * (1 << (2 * t + 2)) * (1 + 2 ** -6) >= M


def _fp32_quotient(x, p):
    """fmaf(x, fl(1/p), 1.5 2^23) - 1.5 2^23 for integer x (int64 array),
    restated exactly in integers: one rounding of the exact x * fl(1/p) +
    1.5 2^23 to FP32, whose spacing there is 1."""
    f32 = np.float32
    pinv = f32(1.0) / f32(p)
    mant, ex = np.frexp(np.float64(pinv))            # pinv = mant 2^ex, mant in [0.5, 1)
    M = int(mant * 2 ** 24)                         # pinv = M 2^(ex - 24), M < 2^24
    sh = 24 - int(ex)                               # x * pinv = x M 2^-sh
    S = x * M + (3 << (22 + sh))                    # (x pinv + 1.5 2^23) 2^sh, exact
    unit = 1 << sh
    low = S % unit
    rounded = S - low + np.where((low > unit // 2) | ((low == unit // 2) & ((S // unit) % 2 == 1)),
                                 unit, 0)
    return rounded // unit - (3 << 22)


def _fp32_residues(mag, neg, p):
    """The split kernel's FP32 residue of sign * mag (mag: non-negative t-bit
    integers, uint64 array; neg: bool array) modulo p: x = sum_d c_d w_d with
    signed 12-bit chunks c_d and w_d = 2^(12 d) mod p in the symmetric range
    (every term and partial sum an exact integer below 2^22.33 in FP32), the
    quotient fmaf(x, fl(1/p), 1.5 2^23) - 1.5 2^23 restated exactly in
    integers (one rounding of the exact x * fl(1/p) + 1.5 2^23 to FP32, whose
    spacing there is 1), and x - q p, with no correction step."""
    sign = np.where(neg, -1, 1).astype(np.int64)
    x = np.zeros(mag.shape, np.int64)
    for d in range(CHUNKS):
        c = ((mag >> np.uint64(CHUNK_BITS * d)) & np.uint64((1 << CHUNK_BITS) - 1)).astype(np.int64)
        w = (1 << (CHUNK_BITS * d)) % p
        w = w - p if w > p // 2 else w
        x += sign * c * w
    assert np.abs(x).max() < 2 ** 22.33
    return x - _fp32_quotient(x, p) * p


def test_fp32_residues_are_exact():
    rng = np.random.default_rng(11)
    t = 60
    mags = [rng.integers(0, 1 << 62, 20000, dtype=np.uint64) >> np.uint64(62 - t)]
    edge = []
    for p in MODULI:                              # values next to multiples of p and p/2
        for base in (p * 12345678901, p * 987654321012345, (1 << t) - 1 - p, p // 2, p):
            edge += [max(0, base + d) for d in range(-3, 4)]
    mags.append(np.array([x % (1 << t) for x in edge], dtype=np.uint64))
    mag = np.concatenate(mags)
    neg = rng.integers(0, 2, mag.size).astype(bool)
    for p in MODULI:
        got = _fp32_residues(mag, neg, p)
        exact = np.array([((v + p // 2) % p) - p // 2 for v in
                          (-int(x) if n else int(x) for x, n in zip(mag, neg))], dtype=np.int64)
        assert np.array_equal(got, exact), p
        assert np.abs(got).max() <= (p - 1) // 2


def test_fp32_quotient_is_exact_next_to_half_integers():
    """Every chunk sum the split can form (|x| < 5 * 4096 * 255) whose
    quotient x / p lies closest to a half-integer (residue +-(p - 1)/2)."""
    lim = CHUNKS * ((1 << CHUNK_BITS) - 1) * 255
    for p in MODULI:
        h = (p - 1) // 2
        q = np.arange(-(lim // p) - 1, lim // p + 2, dtype=np.int64)
        for r in (h, -h):
            x = q * p + r
            x = x[np.abs(x) <= lim]
            assert np.array_equal(_fp32_quotient(x, p), (x - r) // p)


def test_crt_reconstruction_recovers_the_product():
    pairs = crt_table()
    for i, pr in enumerate(pairs):                # each pair's residue is C' mod a b
        for c in (0, 1, -1, 12345678901234567, -98765432109876543):
            y_ref = c % (pr["a"] * pr["b"])
            res = [c % p for p in MODULI]
            u = ((res[2 * i + 1] + 2 * pr["b"] - res[2 * i]) * pr["inv"]) & 0xFFFFFFFF
            t = u - ((u * pr["magic"]) >> 32) * pr["b"]
            assert res[2 * i] + pr["a"] * t == y_ref
    rng = np.random.default_rng(12)
    for k in (64, 1000, 4096):
        t = mod_bits(k)
        lim = k * (1 << (2 * t)) - 1
        vals = [0, 1, -1, lim, -lim, lim // 2, -(lim // 3)]
        vals += [int(x) for x in rng.integers(-(1 << 62), 1 << 62, 300)]
        vals += [(int(a) << 62) + int(b) for a, b in
                 zip(rng.integers(-(lim >> 62), lim >> 62, 300), rng.integers(0, 1 << 62, 300))]
        for c in vals:
            assert abs(c) <= lim
            residues = [c % p for p in MODULI]
            assert reconstruct(residues, pairs) == c


def test_epilogue_reduction_is_exact():
    off_shift = int(re.search(r"off = pm << (\d+)", SRC).group(1))
    magic_shift = int(re.search(r"\(\(1ull << (\d+)\) \+ MODULI\[l\] - 1\) / MODULI\[l\]",
                                SRC).group(1))
    q_shift = int(re.search(r"__umulhi\(u, magic\) >> (\d+)", SRC).group(1))
    assert magic_shift == 32 + q_shift
    assert re.search(r"MOD_K_SEGMENT = 2 \* MAX_K_SEGMENT;", SRC)
    bound = 2 * 4096 * 255 * 255                 # |residue sum| of one 8192-deep segment
    rng = np.random.default_rng(13)
    for p in MODULI:
        magic = ((1 << magic_shift) + p - 1) // p
        assert magic < 1 << 32
        sums = list(range(-bound, -bound + 2000)) + list(range(bound - 2000, bound + 1))
        sums += [int(x) for x in rng.integers(-bound, bound + 1, 20000)]
        for v in sums:
            u = (v + (p << off_shift)) & 0xFFFFFFFF
            assert 0 <= u < 1 << 31
            q = ((u * magic) >> 32) >> q_shift
            assert u - q * p == v % p
