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


def _signed64(x: int) -> int:
    return x - (1 << 64) if x >= (1 << 63) else x


def uniform_device(seed: int, shape, device="cuda", lo: float = -1.0, hi: float = 1.0,
                   chunk: int = 1 << 26):
    """The same numbers as ``uniform`` generated by torch on ``device``.

    Returns a torch float64 tensor holding the column-major matrix as its
    transpose (``out.T`` is ``uniform(seed, shape)``; for a 1-D shape the
    vector itself), so ``out.data_ptr()`` is a column-major buffer with
    leading dimension ``shape[0]``.  The splitmix64 rounds run in int64
    arithmetic (products wrap modulo 2^64, right shifts are masked to be
    logical), in chunks of ``chunk`` elements to bound temporary memory.
    """
    import torch
    shape = tuple(int(s) for s in (shape if isinstance(shape, (tuple, list)) else (shape,)))
    n = int(np.prod(shape))
    gold, m1, m2 = (_signed64(int(c)) for c in (_GOLD, _M1, _M2))
    base = _signed64((seed * (1 << 32)) & 0xFFFFFFFFFFFFFFFF)

    def lshr(z, s):
        return (z >> s) & ((1 << (64 - s)) - 1)

    out = torch.empty(n, dtype=torch.float64, device=device)
    for c0 in range(0, n, chunk):
        cn = min(chunk, n - c0)
        z = torch.arange(c0 + 1, c0 + cn + 1, dtype=torch.int64, device=device) * gold + base
        z = (z ^ lshr(z, 30)) * m1
        z = (z ^ lshr(z, 27)) * m2
        z = z ^ lshr(z, 31)
        u = lshr(z, 11).to(torch.float64) * (2.0 ** -53)
        out[c0:c0 + cn] = lo + (hi - lo) * u
        del z, u
    if len(shape) == 1:
        return out
    return out.view(shape[1], shape[0]) if len(shape) == 2 else out


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
