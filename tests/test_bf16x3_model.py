"""The three-term bf16 split of the tensor-core SGEMM, checked on the CPU.

Each FP32 element x is split as in the split kernel of
openblas_gb300/csrc/sgemm_tc.cu:
- x1 = bf16(x), rounded to nearest even, or toward zero when a finite x
  would round to infinity;
- x2 = bf16(x - x1);
- x3 = bf16(x - x1 - x2).
Each residual is formed in FP32.  Here bf16 rounding is done on the FP32 bit
pattern.  The tests pin the properties that the kernel's accuracy argument
uses:
- the split is exact for |x| >= 2^-110, in every binade up to FLT_MAX;
- |x2| <= 2^-8 |x| (2^-7 where x1 rounds toward zero next to FLT_MAX) and
  |x3| <= 2^-17 |x|;
- the three dropped product terms stay within (2^-24 + 2^-34) |a b|;
- below 2^-110 the loss is as documented: at most 2^-(7 + E) relative for
  FP32 exponent field E >= 1.
"""
from __future__ import annotations

import numpy as np


def bf16_rn(x: np.ndarray) -> np.ndarray:
    u = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def bf16_rz(x: np.ndarray) -> np.ndarray:
    return ((x.astype(np.float32).view(np.uint32) >> 16) << 16).astype(np.uint32).view(np.float32)


def split3(x: np.ndarray):
    with np.errstate(over="ignore", invalid="ignore"):
        x1 = bf16_rn(x)
        x1 = np.where(np.isinf(x1) & np.isfinite(x), bf16_rz(x), x1)
        r = (x - x1).astype(np.float32)
        x2 = bf16_rn(r)
        r2 = (r - x2).astype(np.float32)
        x3 = bf16_rn(r2)
    return x1, x2, x3, r, r2


def _binade(field: int, count: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    man = rng.integers(0, 2 ** 23, size=count, dtype=np.uint64)
    sign = rng.integers(0, 2, size=count, dtype=np.uint64) << np.uint64(31)
    return (sign | (np.uint64(field) << np.uint64(23)) | man).astype(np.uint32).view(np.float32)


def _f64(v):
    return v.astype(np.float64)


def test_parts_are_bf16_and_residuals_exact():
    x = np.concatenate([_binade(f, 20000, f) for f in range(0, 255, 7)])
    x1, x2, x3, r, r2 = split3(x)
    for part in (x1, x2, x3):
        assert np.all((part.view(np.uint32) & 0xFFFF) == 0)   # representable in bf16
        assert np.all(np.isfinite(part))
    assert np.array_equal(_f64(r), _f64(x) - _f64(x1))
    assert np.array_equal(_f64(r2), _f64(r) - _f64(x2))


def test_split_exact_from_2_to_the_minus_110():
    fmax = np.finfo(np.float32).max
    edge = np.array([fmax, -fmax, np.nextafter(fmax, 0, dtype=np.float32), 2.0 ** -110,
                     -(2.0 ** -110), 1.0, -3.0], dtype=np.float32)
    for field in list(range(17, 255)):
        x = np.concatenate([_binade(field, 4000, 1000 + field), edge])
        x1, x2, x3, _, _ = split3(x)
        d = _f64(x) - _f64(x1) - _f64(x2) - _f64(x3)
        assert not d.any(), field
        # x1 rounds toward zero where rounding to nearest would overflow, and
        # may then leave a whole bf16 unit: 2^-7 instead of 2^-8
        with np.errstate(over="ignore"):
            toward_zero = np.isinf(bf16_rn(x))
        bound2 = np.where(toward_zero, 2.0 ** -7, 2.0 ** -8)
        assert np.all(np.abs(_f64(x2)) <= bound2 * np.abs(_f64(x))), field
        assert np.all(np.abs(_f64(x3)) <= 2.0 ** -17 * np.abs(_f64(x))), field


def test_dropped_terms_bound():
    rng = np.random.default_rng(7)
    n = 1_000_000
    a = (rng.uniform(-1, 1, n) * 2.0 ** rng.integers(-50, 50, n)).astype(np.float32)
    b = (rng.uniform(-1, 1, n) * 2.0 ** rng.integers(-50, 50, n)).astype(np.float32)
    a1, a2, a3, _, _ = split3(a)
    b1, b2, b3, _, _ = split3(b)
    kept = (_f64(a1) * _f64(b1) + _f64(a1) * _f64(b2) + _f64(a2) * _f64(b1)
            + _f64(a1) * _f64(b3) + _f64(a3) * _f64(b1) + _f64(a2) * _f64(b2))
    ab = _f64(a) * _f64(b)
    assert np.all(np.abs(ab - kept) <= (2.0 ** -24 + 2.0 ** -34) * np.abs(ab))
    # each kept product of two bf16 values is exact in FP32 (8 + 8 significant bits)
    for p, q in ((a1, b1), (a1, b2), (a2, b1), (a1, b3), (a3, b1), (a2, b2)):
        prod = _f64(p) * _f64(q)
        assert np.array_equal(prod.astype(np.float32).astype(np.float64), prod)


def test_loss_below_2_to_the_minus_110():
    for field in range(1, 17):
        x = _binade(field, 20000, 2000 + field)
        x1, x2, x3, _, _ = split3(x)
        rel = np.abs(_f64(x) - _f64(x1) - _f64(x2) - _f64(x3)) / np.abs(_f64(x))
        assert rel.max() <= 2.0 ** -(7 + field), field
        assert rel.max() > 0, field   # the loss is real, hence the documented limit
