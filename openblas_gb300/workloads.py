"""Seeded synthetic inputs for the level-3 / LAPACK workloads.

The generator is counter-based splitmix64: element ``i`` of stream ``seed``
is ``mix(seed * 2^32 + i)``, so any sub-block can be regenerated without
replaying the stream and the same numbers come out on any host.  Uniform
doubles use the top 53 bits.

Workload shapes follow the benchmark configurations of the level-3 sweep
(uniform(-1,1) operands, padded leading dimensions, a well-conditioned
lower-triangular TRSM operand with diagonal n+U(0,1), exponent-spread
operands U*2^E for the emulated-FP64 GEMM, an SPD matrix B*B^T/n + I for
Cholesky and U*diag(logspace)*V^T for the ill-conditioned solves).
"""
from __future__ import annotations

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Counter-based splitmix64 stream: ``count`` uint64 values."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed * (1 << 32)) & 0xFFFFFFFFFFFFFFFF)
        z = base + (np.arange(offset, offset + count, dtype=np.uint64) + np.uint64(1)) * _GOLD
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, shape, lo: float = -1.0, hi: float = 1.0, offset: int = 0) -> np.ndarray:
    """Uniform [lo, hi) doubles, filled in Fortran (column-major) order."""
    n = int(np.prod(shape))
    u = (splitmix64(seed, n, offset) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    return (lo + (hi - lo) * u).reshape(shape, order="F")


def randint(seed: int, shape, lo: int, hi: int) -> np.ndarray:
    """Integers uniform in [lo, hi] inclusive."""
    n = int(np.prod(shape))
    span = np.uint64(hi - lo + 1)
    return (splitmix64(seed, n) % span).astype(np.int64).reshape(shape, order="F") + lo


def padded(a: np.ndarray, ld: int) -> np.ndarray:
    """Column-major copy of ``a`` embedded in an ld x ncols buffer (ld >= rows)."""
    m, n = a.shape
    buf = np.zeros((ld, n), dtype=a.dtype, order="F")
    buf[:m, :] = a
    return buf


def gemm_operands(seed: int, m: int, n: int, k: int, transa: str = "N", transb: str = "N",
                  pad: int = 0, dtype=np.float64):
    """A, B, C for C = alpha*op(A)*op(B) + beta*C with ld = rows + pad."""
    ra, ca = (m, k) if transa.upper() == "N" else (k, m)
    rb, cb = (k, n) if transb.upper() == "N" else (n, k)
    A = uniform(seed, (ra, ca)).astype(dtype)
    B = uniform(seed + 1, (rb, cb)).astype(dtype)
    C = uniform(seed + 2, (m, n)).astype(dtype)
    if pad:
        A, B, C = padded(A, ra + pad), padded(B, rb + pad), padded(C, m + pad)
    return np.asfortranarray(A), np.asfortranarray(B), np.asfortranarray(C)


def exponent_spread(seed: int, shape, e: int) -> np.ndarray:
    """U .* 2^E with U uniform(-1,1), E integer uniform in [-e, e]."""
    u = uniform(seed, shape)
    if e == 0:
        return u
    E = randint(seed + 7919, shape, -e, e)
    return np.ldexp(u, E)


def trsm_lower(seed: int, n: int) -> np.ndarray:
    """Strictly-lower uniform(-1,1) with diagonal n + U(0,1) (well conditioned)."""
    L = np.tril(uniform(seed, (n, n)), -1)
    d = n + uniform(seed + 3, (n,), 0.0, 1.0)
    L[np.arange(n), np.arange(n)] = d
    return np.asfortranarray(L)


def spd(seed: int, n: int) -> np.ndarray:
    """B*B^T/n + I with B uniform(-1,1)."""
    B = uniform(seed, (n, n))
    return np.asfortranarray(B @ B.T / n + np.eye(n))


def spd_ill_conditioned(seed: int, n: int, kappa_exp: float) -> np.ndarray:
    """U*diag(logspace(0,-kappa))*U^T with U from QR of seeded uniforms (SPD)."""
    U, _ = np.linalg.qr(uniform(seed, (n, n)))
    s = np.logspace(0.0, -float(kappa_exp), n)
    A = (U * s) @ U.T
    return np.asfortranarray((A + A.T) / 2)


def ill_conditioned(seed: int, n: int, kappa_exp: float) -> np.ndarray:
    """U*diag(logspace(0,-kappa))*V^T with U, V from QR of seeded uniforms."""
    U, _ = np.linalg.qr(uniform(seed, (n, n)))
    V, _ = np.linalg.qr(uniform(seed + 1, (n, n)))
    s = np.logspace(0.0, -float(kappa_exp), n)
    return np.asfortranarray((U * s) @ V.T)
